// Many independent BCSR x dense products in one persistent tcgen05 launch.
//
// A plan, built once per batch on the host, holds
//   * a device problem table: per problem its tensor maps (A blocks one at a
//     time and in groups, B panels), its column indices, C, ldc, N, block
//     height and column tile. TMA reads tensor maps from global memory as well
//     as from kernel parameters, so one kernel serves any number of problems;
//   * an item list: one item per (problem, block row, column tile), with the
//     row's block range, ordered heaviest first (longest-processing-time
//     order: a persistent CTA that takes the next item off the queue then
//     finishes the batch with the small items, not with one long row);
//   * the work queue: {next item, CTAs done}. The last CTA of a launch zeroes
//     it again, so the launch can be replayed as is (from a CUDA graph).
//
// The kernel is the single-product tcgen05 pipeline with the block height and
// the column tile read per item instead of fixed at compile time: the UMMA's
// N field, the A box height, the epilogue's row loop and the panel width all
// come from the item's problem. Shared-memory slots are sized for the largest
// case (64-row blocks, 256-column panels), TMEM for two 128-column x 64-row
// accumulators. The lead warp copies each item's problem fields into the item
// ring in shared memory, so the other roles never read the problem table.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>
#include "internal.h"
#include "ptx.cuh"
#include "spmm_mma.cuh"
#include "tcgen05.cuh"

namespace spmm {
namespace {

struct alignas(64) BatchProblemDev {
  CUtensorMap tmA1;   // A values as [rows x 16], box = one block (a stacked problem: one member block)
  CUtensorMap tmAg;   // same tensor, box = G blocks (not used by a stacked problem)
  CUtensorMap tmB;    // B panels: 3-D {64, K, N/64} box {64, 16, ntp/64}, or 2-D box {64, 16}
  const int* col_idx;
  float* C;
  long long ldc;
  int N, bR, ntp, panel3d;
  // stacked problem (stk > 1): its 64-row blocks are assembled in shared
  // memory from stk member blocks of mbR rows each; smap holds, per stacked
  // block and member, the source block of A or -1 (rows of zeros, loaded
  // from row oob_row, past the end of A's tensor map)
  const int* smap;
  int stk, mbR, oob_row, pad;
};

struct BatchItem {
  int prob, br, nt, start;
  int end, pad0, pad1, pad2;
};

struct BatchParams {
  const BatchProblemDev* probs;
  const BatchItem* items;
  int n_items;
  unsigned* queue;
  unsigned* err;
  unsigned long long timeout_ns;
};

// One entry of the item ring (64 bytes): the item plus the problem fields the
// consumer roles need. prob < 0 ends the stream.
struct RingRec {
  int prob, br, nt, start, end, bR, ntp, N, panel3d, stk;
  const int* col_idx;
  float* C;
  long long ldc;
};
static_assert(sizeof(RingRec) == 64, "ring record");

constexpr int kBatchThreads = 352;   // 11 warps, the roles of the single-product pipeline
constexpr int kMaxBR = 64, kMaxNT = 256;

template <int STAGES, int G>
struct BatchCfg {
  static constexpr int kBoxBytes = 16 * 128;
  static constexpr int kPanelBytes = (kMaxNT / 64) * kBoxBytes;   // slot stride of one panel
  static constexpr int kAStage = ((G * kMaxBR * 32 + 1023) / 1024) * 1024;
  static constexpr int kStage = kAStage + G * kPanelBytes;
  static constexpr int kAccCols = (kMaxNT / 128) * kMaxBR;          // 128
  static constexpr int kTmemCols = 2 * kAccCols;                     // two accumulators
  static constexpr int kQ = 4;
  static constexpr size_t kSmem = 1024 + (size_t)STAGES * kStage + 1024;
  static_assert(G * kMaxBR <= 256 && 32 % G == 0, "a group is one TMA box and never straddles an index chunk");
};

template <int STAGES, int G, bool BF16>
__global__ void __launch_bounds__(kBatchThreads, 2) k_bcsr_tc_batch(const BatchParams p) {
  using Cfg = BatchCfg<STAGES, G>;
  constexpr int kQ = Cfg::kQ;
  constexpr int kBIssuers = 4;
  constexpr int kIssuers = 2;   // UMMA issuers: warp 1 (slice 0) and warp 10 (slice 1)
  // kind::f16 instruction descriptor without N: D f32, A MN-major, B K-major, M = 128
  constexpr uint32_t kIdescBase = (1u << 4) | ((BF16 ? 1u : 0u) << 7) | ((BF16 ? 1u : 0u) << 10) |
                                  (1u << 15) | ((uint32_t)(128 >> 4) << 24);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)STAGES * Cfg::kStage);
  // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], done, qfull[kQ], qempty[kQ];
  // then the TMEM address and the item ring
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES;
  const uint32_t tfull0 = empty0 + 8 * STAGES, tempty0 = tfull0 + 16, done_bar = tempty0 + 16;
  const uint32_t qfull0 = done_bar + 8, qempty0 = qfull0 + 8 * kQ;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5 + 2 * kQ);
  RingRec* ring = reinterpret_cast<RingRec*>(reinterpret_cast<uint8_t*>(bars) + 512);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 32) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, kIssuers);   // each MMA issuer's commit
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull0 + 8 * b, kIssuers);
      mbar_init(tempty0 + 8 * b, 4);
    }
    mbar_init(done_bar, kIssuers);
    for (int q = 0; q < kQ; ++q) {
      mbar_init(qfull0 + 8 * q, 1);
      mbar_init(qempty0 + 8 * q, kIssuers + kBIssuers + 4);   // MMA issuers, B issuers, epilogue warps
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

  // Ring entry `it`, read by a whole warp: lane 0 waits (bounded), every lane
  // copies the record, lane 0 releases the entry. False on a timeout.
  auto read_rec_warp = [&](uint32_t it, RingRec& rec, unsigned code) -> bool {
    const uint32_t q = it % kQ;
    int ok = 1;
    if (lane == 0 && !mbar_wait(qfull0 + 8 * q, (it / kQ) & 1, p.timeout_ns)) {
      atomicOr(p.err, code);
      ok = 0;
    }
    if (!__shfl_sync(0xffffffffu, ok, 0)) return false;
    __syncwarp();
    rec = ring[q];
    __syncwarp();
    if (lane == 0) mbar_arrive(qempty0 + 8 * q);
    return true;
  };
  const int bidx = warp == 2 ? 0 : warp == 3 ? 1 : warp == 8 ? 2 : warp == 9 ? 3 : -1;

  if (warp == 0) {
    // ------------------------------ lead producer ----------------------------------
    if (lane == 0) {
      const uint64_t pol_a = l2_policy_evict_first();
      auto fetch = [&](RingRec& r) {
        const int idx = (int)atomicAdd(p.queue, 1u);
        if (idx >= p.n_items) {
          r.prob = -1;
          return;
        }
        const int4 a = __ldg(reinterpret_cast<const int4*>(p.items + idx));
        const int4 b = __ldg(reinterpret_cast<const int4*>(p.items + idx) + 1);
        r.prob = a.x;
        r.br = a.y;
        r.nt = a.z;
        r.start = a.w;
        r.end = b.x;
        const BatchProblemDev* pr = p.probs + r.prob;
        r.bR = __ldg(&pr->bR);
        r.ntp = __ldg(&pr->ntp);
        r.N = __ldg(&pr->N);
        r.panel3d = __ldg(&pr->panel3d);
        r.stk = __ldg(&pr->stk);
        r.col_idx = pr->col_idx;
        r.C = pr->C;
        r.ldc = __ldg(&pr->ldc);
        if (r.end > r.start) {
          if (r.stk <= 1) tma_prefetch_desc(&pr->tmAg);
          tma_prefetch_desc(&pr->tmB);
        }
      };
      uint32_t gs = 0, it = 0;
      bool failed = false;
      RingRec cur;
      fetch(cur);
      for (;; ++it) {
        const uint32_t q = it % kQ;
        if (it >= (uint32_t)kQ && !mbar_wait(qempty0 + 8 * q, ((it / kQ) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 4u);
          failed = true;
        }
        if (failed) cur.prob = -1;
        ring[q] = cur;
        mbar_arrive(qfull0 + 8 * q);
        if (cur.prob < 0) break;
        RingRec nxt;
        fetch(nxt);
        const BatchProblemDev* pr = p.probs + cur.prob;
        const int bR = cur.bR;
        const uint32_t blk_bytes = (uint32_t)(bR * 32 + cur.ntp * 32);
        for (int j0 = cur.start; j0 < cur.end; j0 += G, ++gs) {
          const int n = min(G, cur.end - j0);
          const int s = (int)(gs % STAGES);
          if (gs >= (uint32_t)STAGES && !mbar_wait(empty0 + 8 * s, ((gs / STAGES) + 1) & 1, p.timeout_ns)) {
            atomicOr(p.err, 4u);
            failed = true;
            break;
          }
          const uint32_t fb = full0 + 8 * s;
          mbar_arrive_expect_tx(fb, (uint32_t)n * blk_bytes);
          uint8_t* a_dst = smem + (size_t)s * Cfg::kStage;
          const int y0 = j0 * bR;
          if (cur.stk > 1) {
            // a stacked problem's member blocks are copied by the B issuers
          } else if (n == G) {
            tma_tile_2d_g2s(smem_u32(a_dst), &pr->tmAg, 0, y0, fb, pol_a);
          } else {
            for (int b = 0; b < n; ++b)
              tma_tile_2d_g2s(smem_u32(a_dst + b * bR * 32), &pr->tmA1, 0, y0 + b * bR, fb, pol_a);
          }
        }
        if (failed) {
          // publish the end of the stream in the next ring entry
          continue;
        }
        cur = nxt;
      }
      // the last CTA to finish resets the queue for the next launch
      __threadfence();
      if (atomicAdd(p.queue + 1, 1u) == gridDim.x - 1) {
        p.queue[0] = 0;
        p.queue[1] = 0;
        __threadfence();
      }
    }
    __syncwarp();
  } else if (bidx >= 0) {
    // ------------------------------ B-panel issuers ----------------------------------
    const uint64_t pol_b = l2_policy_evict_last();
    uint32_t gs = 0;
    int failed = 0;
    for (uint32_t it = 0; !failed; ++it) {
      RingRec rec;
      if (!read_rec_warp(it, rec, 4u) || rec.prob < 0) break;
      const BatchProblemDev* pr = p.probs + rec.prob;
      const CUtensorMap* tmB = &pr->tmB;
      const int boxes = rec.ntp / 64;
      // One pass over the item's blocks. A stacked problem (stk > 1) also
      // copies, per stacked block, its stk member blocks of mbR rows from the
      // source blocks its map names (-1: a box past the end of A, which reads
      // zeros). The two cases are separate instantiations, so the plain path
      // carries none of the member bookkeeping.
      auto issue_blocks = [&](auto stacked_tag) {
        constexpr bool kStacked = decltype(stacked_tag)::value;
        const int stk = rec.stk;
        const int* smap = kStacked ? pr->smap : nullptr;
        const int mbR = kStacked ? __ldg(&pr->mbR) : 0, oob = kStacked ? __ldg(&pr->oob_row) : 0;
        auto load_members = [&](int j, int (&mm)[4]) {
#pragma unroll
          for (int t = 0; t < 4; ++t) mm[t] = (t < stk && j < rec.end) ? __ldg(smap + (long long)j * stk + t) : -1;
        };
        int mym[4] = {-1, -1, -1, -1};
        if constexpr (kStacked) load_members(rec.start + lane, mym);
        int mycol = lane < rec.end - rec.start ? __ldg(rec.col_idx + rec.start + lane) : 0;
        for (int base = rec.start; base < rec.end && !failed; base += 32) {
          const int cnt = min(32, rec.end - base);
          const int cur = mycol;
          int curm[4] = {mym[0], mym[1], mym[2], mym[3]};
          if constexpr (kStacked)
            if (base + 32 < rec.end) load_members(base + 32 + lane, mym);
          if (base + 32 < rec.end) mycol = lane < rec.end - base - 32 ? __ldg(rec.col_idx + base + 32 + lane) : 0;
          for (int i0 = 0; i0 < cnt; i0 += G, ++gs) {
            const int n = min(G, cnt - i0);
            const int s = (int)(gs % STAGES);
            // Wait for the slot only in groups this issuer copies into: such a
            // group cannot be released without its bytes, so the slot's empty
            // barrier is at most one phase ahead. (An issuer that also waited in
            // groups it has no block in could fall two phases behind and miss a
            // parity flip.)
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
              int src[4] = {-1, -1, -1, -1};
              if constexpr (kStacked) {
#pragma unroll
                for (int t = 0; t < 4; ++t) src[t] = __shfl_sync(0xffffffffu, curm[t], i0 + b);
              }
              if (lane == 0) {
                const uint32_t fb = full0 + 8 * s;
                if constexpr (kStacked) {
                  // the stacked 64-row block: member t's rows at t * mbR
                  uint8_t* a_dst = smem + (size_t)s * Cfg::kStage + (size_t)b * 64 * 32;
#pragma unroll
                  for (int t = 0; t < 4; ++t)
                    if (t < stk)
                      tma_tile_2d_g2s(smem_u32(a_dst + t * mbR * 32), &pr->tmA1, 0, src[t] >= 0 ? src[t] * mbR : oob,
                                      fb, pol_b);
                }
                uint8_t* b_dst = b_dst0 + (size_t)b * Cfg::kPanelBytes;
                if (rec.panel3d) {
                  tma_tile_3d_g2s(smem_u32(b_dst), tmB, 0, col * 16, rec.nt * boxes, fb, pol_b);
                } else {
                  for (int bx = 0; bx < boxes; ++bx)
                    tma_tile_2d_g2s(smem_u32(b_dst + bx * Cfg::kBoxBytes), tmB, rec.nt * rec.ntp + bx * 64,
                                    col * 16, fb, pol_b);
                }
              }
            }
          }
        }
      };
      if (rec.stk > 1)
        issue_blocks(std::true_type{});
      else
        issue_blocks(std::false_type{});
    }
  } else if (warp == 1 || warp == 10) {
    // ------------------------------ MMA issuers ----------------------------------
    // Warp 1 issues slice 0 of every block and warp 10 slice 1 of a 256-column
    // item (disjoint accumulators; for a 128-column item it only commits): one
    // thread's UMMA issue rate is close to the critical path. Each commits to
    // the slot, accumulator and done barriers, which expect one commit per issuer.
    if (lane == 0) {
      const int mi = warp == 1 ? 0 : 1;
      uint32_t gs = 0, it = 0;
      bool failed = false;
      for (;; ++it) {
        const uint32_t q = it % kQ;
        if (!mbar_wait(qfull0 + 8 * q, (it / kQ) & 1, p.timeout_ns)) {
          atomicOr(p.err, 8u);
          break;
        }
        const RingRec rec = ring[q];
        mbar_arrive(qempty0 + 8 * q);
        if (rec.prob < 0) break;
        const int bR = rec.bR, J = rec.ntp / 128;
        const uint32_t idesc = kIdescBase | ((uint32_t)(bR >> 3) << 17);
        const uint32_t acc = it & 1;
        if (it >= 2u && !mbar_wait(tempty0 + 8 * acc, ((it / 2) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 8u);
          break;
        }
        tc_fence_after();
        const uint32_t d0 = tmem + acc * Cfg::kAccCols;
        for (int j0 = rec.start; j0 < rec.end; j0 += G, ++gs) {
          const int n = min(G, rec.end - j0);
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
            const uint32_t b_addr = b_slot + b * Cfg::kPanelBytes;
            const uint64_t blk = smem_desc(a_slot + b * bR * 32, 16, 256, kLayoutSW32);
            const uint32_t accum = (j0 + b != rec.start) ? 1u : 0u;
            if (mi < J) {
              const uint64_t pan = smem_desc(b_addr + mi * 2 * Cfg::kBoxBytes, 2048, 1024, kLayoutSW128);
              umma_f16(d0 + mi * bR, pan, blk, idesc, accum);
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
    const int q4 = warp & 3;
    for (uint32_t it = 0;; ++it) {
      RingRec rec;
      if (!read_rec_warp(it, rec, 16u) || rec.prob < 0) break;
      const uint32_t acc = it & 1;
      int ok = 1;
      if (lane == 0 && !mbar_wait(tfull0 + 8 * acc, (it / 2) & 1, p.timeout_ns)) {
        atomicOr(p.err, 16u);
        ok = 0;
      }
      if (!__shfl_sync(0xffffffffu, ok, 0)) break;
      __syncwarp();
      tc_fence_after();
      const bool empty = rec.start == rec.end;
      const int bR = rec.bR, J = rec.ntp / 128;
      const long long row0 = (long long)rec.br * bR;
#pragma unroll 1
      for (int j = 0; j < J; ++j) {
        const int n = rec.nt * rec.ntp + j * 128 + q4 * 32 + lane;
        float* cptr = rec.C + row0 * rec.ldc + n;
        const uint32_t taddr = tmem + ((uint32_t)(q4 * 32) << 16) + acc * Cfg::kAccCols + j * bR;
#pragma unroll 1
        for (int c0 = 0; c0 < bR; c0 += 16) {
          float v[16];
          if (!empty) {
            tmem_ld16(taddr + c0, v);
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = 0.f;
          }
          if (n < rec.N) {
#pragma unroll
            for (int i = 0; i < 16; ++i) __stcs(cptr + (long long)(c0 + i) * rec.ldc, v[i]);
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

using BatchFn = void (*)(const BatchParams);
struct BatchEntry {
  int stages, group;
  bool bf16;
  BatchFn fn;
  size_t smem;
};
#define SPMM_BATCH_ENTRY(ST, G, BF) \
  BatchEntry{ST, G, BF, &k_bcsr_tc_batch<ST, G, BF>, BatchCfg<ST, G>::kSmem}
// (ring depth in groups, blocks per group); the first entry per type is the default,
// and the 4-stage one the default of a batch with stacked problems. All three hold
// eight blocks in flight; two groups of four take half the barrier round trips of
// four groups of two and ran the 64-product uneven batch faster with stacking off
// (188 against 192 us); with stacking on, four groups of two ran it in 151 against
// 157 us (and a second seed's 64 products in 257 against 274 us).
const BatchEntry kBatchEntries[] = {
    SPMM_BATCH_ENTRY(2, 4, false), SPMM_BATCH_ENTRY(4, 2, false), SPMM_BATCH_ENTRY(8, 1, false),
    SPMM_BATCH_ENTRY(2, 4, true),  SPMM_BATCH_ENTRY(4, 2, true),  SPMM_BATCH_ENTRY(8, 1, true),
};

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace
}  // namespace spmm

using namespace spmm;

struct spmm_batch_plan {
  int device = -1;
  int count = 0;
  int n_items = 0;
  int grid = 0;
  const BatchEntry* entry = nullptr;
  BatchProblemDev* d_probs = nullptr;
  BatchItem* d_items = nullptr;
  unsigned* d_queue = nullptr;
  unsigned* err = nullptr;
  unsigned long long timeout_ns = 0;
  // 16- and 32-row problems whose block rows share most columns, stacked into
  // 64-row blocks (as a per-matrix plan stacks them): the device arrays of
  // their stacked structure, which the plan owns
  std::vector<void*> owned;
  int stacked = 0;
};

namespace {

spmm_status check_problem(const spmm_problem& pb, int i, spmm_dtype dtype) {
  const std::string at = "problem " + std::to_string(i) + ": ";
  const spmm_bcsr_desc& A = pb.A;
  if (A.dtype != dtype) return fail(SPMM_ERR_INVALID_ARG, at + "all problems must share one dtype");
  if (A.M < 0 || A.K < 0 || pb.N < 0) return fail(SPMM_ERR_INVALID_ARG, at + "negative size");
  if (A.bC != 16) return fail(SPMM_ERR_UNSUPPORTED, at + "block width must be 16");
  if (A.bR != 16 && A.bR != 32 && A.bR != 64)
    return fail(SPMM_ERR_UNSUPPORTED, at + "block height must be 16, 32 or 64");
  if (A.M % A.bR) return fail(SPMM_ERR_INVALID_ARG, at + "M must be a multiple of the block height");
  if (A.K % 16) return fail(SPMM_ERR_INVALID_ARG, at + "K must be a multiple of 16");
  if (A.M == 0 || pb.N == 0) return SPMM_OK;
  if (!A.row_ptr || !pb.C || !pb.B.data) return fail(SPMM_ERR_INVALID_ARG, at + "null pointer");
  if (pb.N % 8) return fail(SPMM_ERR_UNSUPPORTED, at + "N must be a multiple of 8");
  if (pb.B.ldb < pb.N || pb.B.ldb % 8) return fail(SPMM_ERR_MISALIGNED, at + "ldb must be >= N and a multiple of 8");
  if (pb.ldc < pb.N || pb.ldc % 4) return fail(SPMM_ERR_MISALIGNED, at + "ldc must be >= N and a multiple of 4");
  if (!aligned16(A.vals) || !aligned16(pb.B.data) || !aligned16(pb.C))
    return fail(SPMM_ERR_MISALIGNED, at + "A values, B and C must be 16-byte aligned");
  return SPMM_OK;
}

void free_plan(spmm_batch_plan* p) {
  if (!p) return;
  if (p->d_probs) cudaFree(p->d_probs);
  if (p->d_items) cudaFree(p->d_items);
  if (p->d_queue) cudaFree(p->d_queue);
  for (void* q : p->owned) cudaFree(q);
  delete p;
}

}  // namespace

extern "C" {

spmm_status spmm_batch_plan_create(const spmm_problem* problems, int count, const spmm_config* cfg,
                                   spmm_batch_plan** plan_out) {
  if (!plan_out) return fail(SPMM_ERR_INVALID_ARG, "null plan_out");
  *plan_out = nullptr;
  if (count < 0 || (count > 0 && !problems)) return fail(SPMM_ERR_INVALID_ARG, "bad problem list");
  spmm_config c;
  std::memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if (c.n_tile != 0 && c.n_tile != 128 && c.n_tile != 256)
    return fail(SPMM_ERR_UNSUPPORTED, "batched launch: n_tile must be 0, 128 or 256");
  const spmm_dtype dtype = count > 0 ? problems[0].A.dtype : SPMM_F16;
  if (dtype != SPMM_F16 && dtype != SPMM_BF16)
    return fail(SPMM_ERR_UNSUPPORTED, "batched launch: fp16 or bf16 problems only");
  for (int i = 0; i < count; ++i) {
    spmm_status st = check_problem(problems[i], i, dtype);
    if (st != SPMM_OK) return st;
  }
  const BatchEntry* e = nullptr;
  for (const BatchEntry& x : kBatchEntries) {
    if (x.bf16 != (dtype == SPMM_BF16)) continue;
    if (c.stages > 0 && x.stages != c.stages) continue;
    e = &x;
    break;
  }
  if (!e) return fail(SPMM_ERR_UNSUPPORTED, "batched launch: stages must be 0, 2, 4 or 8");

  spmm_batch_plan* plan = new spmm_batch_plan();
  plan->count = count;
  plan->entry = e;
  plan->timeout_ns = wait_limit_ns();
  if (cudaGetDevice(&plan->device) != cudaSuccess) {
    delete plan;
    return fail(SPMM_ERR_CUDA, "no current device");
  }
  plan->err = device_error_word();
  if (!plan->err) {
    delete plan;
    return fail(SPMM_ERR_CUDA, "could not set up the device error word");
  }

  // Host copies of the row pointers (one synchronous read per problem) give
  // every item its block range and cost.
  std::vector<BatchProblemDev> probs(count > 0 ? count : 1);
  std::memset(probs.data(), 0, sizeof(BatchProblemDev) * probs.size());
  struct Keyed {
    double cost;
    BatchItem it;
  };
  std::vector<Keyed> items;
  std::vector<int> rp;
  // the group maps (box = G blocks) of the problems that are not stacked,
  // encoded once the ring's group size is known
  struct GroupMap {
    int prob;
    const void* vals;
    unsigned long long rows;
    int bR;
  };
  std::vector<GroupMap> group_maps;
  cudaError_t ce = cudaSuccess;
  for (int i = 0; i < count; ++i) {
    const spmm_problem& pb = problems[i];
    const spmm_bcsr_desc& A = pb.A;
    if (A.M == 0 || pb.N == 0) continue;
    const int MB = A.M / A.bR;
    rp.resize(MB + 1);
    cudaError_t ce = cudaMemcpy(rp.data(), A.row_ptr, sizeof(int) * (MB + 1), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) {
      free_plan(plan);
      return cuda_fail(ce, "reading row_ptr");
    }
    if (rp[0] != 0) {
      free_plan(plan);
      return fail(SPMM_ERR_BAD_STRUCTURE, "problem " + std::to_string(i) + ": row_ptr[0] != 0");
    }
    for (int r = 0; r < MB; ++r)
      if (rp[r + 1] < rp[r] || rp[r + 1] - rp[r] > A.K / 16) {
        free_plan(plan);
        return fail(SPMM_ERR_BAD_STRUCTURE, "problem " + std::to_string(i) + ": row_ptr not monotone or a row too long");
      }
    const long long nnzb = rp[MB];
    if (nnzb > 0 && !A.col_idx) {
      free_plan(plan);
      return fail(SPMM_ERR_INVALID_ARG, "problem " + std::to_string(i) + ": null col_idx");
    }
    const int ntp = c.n_tile > 0 ? c.n_tile : (pb.N <= 128 ? 128 : 256);
    BatchProblemDev& d = probs[i];
    d.col_idx = A.col_idx;
    d.C = pb.C;
    d.ldc = pb.ldc;
    d.N = pb.N;
    d.bR = A.bR;
    d.ntp = ntp;
    // Stacking: 16- or 32-row block rows that make up 64 rows of C are run as
    // one 64-row row over the union of their block columns (zeros where a row
    // has no block), when that union holds at most 60 % of the blocks: one
    // UMMA, one B panel and one item for up to 4 blocks.
    int bR_run = A.bR, rows_run = MB;
    if ((A.bR == 16 || A.bR == 32) && A.M % 64 == 0 && nnzb > 0 && A.vals) {
      std::vector<int> ci((size_t)nnzb), srp, sci, smap;
      ce = cudaMemcpy(ci.data(), A.col_idx, sizeof(int) * nnzb, cudaMemcpyDeviceToHost);
      if (ce != cudaSuccess) {
        free_plan(plan);
        return cuda_fail(ce, "reading col_idx");
      }
      const int stk = 64 / A.bR;
      if (stack_structure_host(rp.data(), ci.data(), MB, stk, &srp, &sci, &smap) &&
          (long long)sci.size() * 100 <= nnzb * 60) {
        int* d_sci = nullptr;
        int* d_map = nullptr;
        ce = cudaMalloc(&d_sci, sizeof(int) * sci.size());
        if (ce == cudaSuccess) plan->owned.push_back(d_sci), ce = cudaMalloc(&d_map, sizeof(int) * smap.size());
        if (ce == cudaSuccess) plan->owned.push_back(d_map);
        if (ce == cudaSuccess) ce = cudaMemcpy(d_sci, sci.data(), sizeof(int) * sci.size(), cudaMemcpyHostToDevice);
        if (ce == cudaSuccess)
          ce = cudaMemcpy(d_map, smap.data(), sizeof(int) * smap.size(), cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) {
          free_plan(plan);
          return cuda_fail(ce, "setting up a stacked problem");
        }
        plan->stacked += 1;
        rp.assign(srp.begin(), srp.end());
        rows_run = (int)srp.size() - 1;
        bR_run = 64;
        d.col_idx = d_sci;
        d.bR = 64;
        d.smap = d_map;
        d.stk = stk;
        d.mbR = A.bR;
      }
    }
    if (nnzb > 0) {
      // A's values as [rows x 16]; a stacked problem reads its member blocks
      // (mbR rows) from the original values, and rows past rows_bound read zeros
      const int box_rows = d.stk > 1 ? d.mbR : bR_run;
      const unsigned long long rows_bound =
          std::max<unsigned long long>((unsigned long long)MB * (A.K / 16) * A.bR, 256ull);
      d.oob_row = (int)rows_bound;
      spmm_status st = rows_bound >= (1ull << 31) - 64
                           ? fail(SPMM_ERR_UNSUPPORTED, "A too large for the tcgen05 pipeline")
                           : encode_tile_map_2d(&d.tmA1, CU_TENSOR_MAP_DATA_TYPE_UINT16, A.vals, 16, rows_bound,
                                                32, 16, (uint32_t)box_rows, CU_TENSOR_MAP_SWIZZLE_32B);
      if (st == SPMM_OK && d.stk <= 1) group_maps.push_back(GroupMap{i, A.vals, rows_bound, A.bR});
      d.panel3d = pb.N % 64 == 0 ? 1 : 0;
      if (st == SPMM_OK && d.panel3d &&
          encode_panel_map_3d(&d.tmB, pb.B.data, (uint64_t)pb.N, (uint64_t)A.K, (uint64_t)pb.B.ldb * 2,
                              (uint32_t)(ntp / 64)) != SPMM_OK)
        d.panel3d = 0;
      if (st == SPMM_OK && !d.panel3d)
        st = encode_tile_map_2d(&d.tmB, CU_TENSOR_MAP_DATA_TYPE_UINT16, pb.B.data, (uint64_t)pb.N,
                                (uint64_t)A.K, (uint64_t)pb.B.ldb * 2, 64, 16, CU_TENSOR_MAP_SWIZZLE_128B);
      if (st != SPMM_OK) {
        free_plan(plan);
        return st;
      }
    }
    const int ntiles = (pb.N + ntp - 1) / ntp;
    // cost of an item ~ bytes it moves: per block the A block and a B panel,
    // plus the C tile it writes
    for (int r = 0; r < rows_run; ++r) {
      const int nb = rp[r + 1] - rp[r];
      for (int t = 0; t < ntiles; ++t) {
        Keyed k;
        k.cost = (double)nb * (bR_run * 32 + ntp * 32) + (double)bR_run * ntp * 4;
        k.it = BatchItem{i, r, t, rp[r], rp[r + 1], 0, 0, 0};
        items.push_back(k);
      }
    }
  }
  if (items.size() >= (1ull << 31) - (1ull << 20)) {
    free_plan(plan);
    return fail(SPMM_ERR_UNSUPPORTED, "batched launch: too many items");
  }
  // A batch with stacked problems defaults to four groups of two: each stacked
  // block is up to four member copies, and the deeper ring keeps more of them
  // in flight.
  if (c.stages == 0 && plan->stacked > 0)
    for (const BatchEntry& x : kBatchEntries)
      if (x.bf16 == e->bf16 && x.stages == 4) e = &x;
  plan->entry = e;
  for (const GroupMap& g : group_maps) {
    spmm_status st = encode_tile_map_2d(&probs[g.prob].tmAg, CU_TENSOR_MAP_DATA_TYPE_UINT16, g.vals, 16, g.rows, 32,
                                        16, (uint32_t)(e->group * g.bR), CU_TENSOR_MAP_SWIZZLE_32B);
    if (st != SPMM_OK) {
      free_plan(plan);
      return st;
    }
  }
  std::stable_sort(items.begin(), items.end(), [](const Keyed& a, const Keyed& b) { return a.cost > b.cost; });
  plan->n_items = (int)items.size();
  std::vector<BatchItem> flat(items.size());
  for (size_t k = 0; k < items.size(); ++k) flat[k] = items[k].it;

  ce = cudaMalloc(&plan->d_probs, sizeof(BatchProblemDev) * probs.size());
  if (ce == cudaSuccess)
    ce = cudaMemcpy(plan->d_probs, probs.data(), sizeof(BatchProblemDev) * probs.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMalloc(&plan->d_items, sizeof(BatchItem) * std::max<size_t>(flat.size(), 1));
  if (ce == cudaSuccess && !flat.empty())
    ce = cudaMemcpy(plan->d_items, flat.data(), sizeof(BatchItem) * flat.size(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMalloc(&plan->d_queue, 2 * sizeof(unsigned));
  if (ce == cudaSuccess) ce = cudaMemset(plan->d_queue, 0, 2 * sizeof(unsigned));
  if (ce == cudaSuccess)
    ce = cudaFuncSetAttribute(reinterpret_cast<const void*>(e->fn), cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)e->smem);
  if (ce != cudaSuccess) {
    free_plan(plan);
    return cuda_fail(ce, "setting up the batch plan");
  }
  // CTAs per SM: TMEM (256 of 512 columns each), shared memory, and the two
  // CTAs the launch bounds budget registers for.
  int smem_sm = 0;
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, plan->device);
  int per_sm = std::min(2, std::max(1, smem_sm / (int)(e->smem + 1024)));
  if (c.ctas_per_sm > 0 && c.ctas_per_sm < per_sm) per_sm = c.ctas_per_sm;
  long long grid = (long long)sm_count() * per_sm;
  if (grid > plan->n_items) grid = plan->n_items;
  plan->grid = (int)grid;
  if (std::getenv("SPMM_DEBUG"))
    std::fprintf(stderr, "[spmm] batch problems=%d stacked=%d items=%d stages=%d group=%d smem=%zu grid=%d\n",
                 count, plan->stacked, plan->n_items, e->stages, e->group, e->smem, plan->grid);
  *plan_out = plan;
  return SPMM_OK;
}

spmm_status spmm_batch_run(const spmm_batch_plan* plan, void* stream) {
  if (!plan) return fail(SPMM_ERR_INVALID_ARG, "null plan");
  int dev = -1;
  SPMM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != plan->device) return fail(SPMM_ERR_INVALID_ARG, "plan was built on another device");
  if (plan->n_items == 0) return SPMM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BatchParams p;
  p.probs = plan->d_probs;
  p.items = plan->d_items;
  p.n_items = plan->n_items;
  p.queue = plan->d_queue;
  p.err = plan->err;
  p.timeout_ns = plan->timeout_ns;
  SPMM_CUDA_TRY(launch_kernel(plan->entry->fn, dim3((unsigned)plan->grid), dim3(kBatchThreads), plan->entry->smem,
                              s, p));
  return SPMM_OK;
}

spmm_status spmm_batch_plan_info(const spmm_batch_plan* plan, int* items, int* stacked_problems) {
  if (!plan) return fail(SPMM_ERR_INVALID_ARG, "null plan");
  if (items) *items = plan->n_items;
  if (stacked_problems) *stacked_problems = plan->stacked;
  return SPMM_OK;
}

spmm_status spmm_batch_plan_destroy(spmm_batch_plan* plan) {
  free_plan(plan);
  return SPMM_OK;
}

}  // extern "C"
