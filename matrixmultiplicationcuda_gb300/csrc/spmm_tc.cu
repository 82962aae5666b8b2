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
//   * the B row-panel (16 rows x NT columns) as 64-column atoms with 128-byte
//     swizzle -- the MMA's A operand in the MN-major canonical layout (8-row
//     groups 1024 B apart, 64-column atoms 2048 B apart); one 3-D copy per
//     panel when N % 64 == 0;
//   * the A blocks (bR rows x 16) with 32-byte swizzle -- the MMA's B operand
//     in the K-major canonical layout (8-row groups 256 B apart); the blocks
//     of a group are contiguous in memory and arrive in one copy.
//
// Warp roles (11 warps, two CTAs per SM): warp 0 takes items (static stride,
// or from a work queue a few groups before the current item is copied),
// publishes them through an item ring and copies A groups;
// warps 2, 3, 8, 9 copy the B panels (a TMA instruction holds its issuing
// thread for ~200 ns, so four threads share them); warp 1 (one thread) issues
// the UMMAs -- with warp 10 taking half of each block's 128-column slices when
// there are two or more -- releases each group's
// ring slot with tcgen05.commit and hands finished accumulators to the
// epilogue; warp 2 owns the TMEM allocation;
// warps 4-7 drain TMEM (double-buffered, so the next item's MMAs overlap) with
// tcgen05.ld and store C with streaming stores. Items = (block row, NT-column
// tile). Every mbarrier wait is bounded; a wait that gives up sets the device
// error word, all roles leave their loops, and the allocating warp frees TMEM
// after the MMA thread has drained its commits.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include "csr.cuh"
#include "internal.h"
#include "ptx.cuh"
#include "spmm_mma.cuh"
#include "tcgen05.cuh"

namespace spmm {
namespace {

struct TcParams {
  const int* row_ptr;
  const int* col_idx;
  const uint8_t* avals;   // A's values (bytes): e4m3 bulk copies, L2 prefetch of an item's blocks
  float* C;
  long long ldc;
  int N;
  int ntiles;
  int n_items;
  unsigned long long timeout_ns;
  unsigned* err;
  int panel3d;      // B panel loaded by one 3-D copy (N % 64 == 0)
  unsigned* queue;  // [0] next item, [1] CTAs done; NULL = static item striding
  int claim_ahead;  // work queue: claim the next item when this many groups of the current one are left to copy
  int inputs_ready; // no kernel earlier on the stream writes A or B (see the dependency wait below)
  int split;        // items per (block row, column tile); > 1: partial sums added into C
  // hybrid (BCSR + CSR): the CSR part's entries are added in the epilogue
  // (NULL csr_row_ptr = plain BCSR)
  const int* csr_row_ptr;
  const int* csr_col_idx;
  const __half* csr_vals;
  const __half* Bh;
  long long ldb;
  // planned hybrid product: a block with col_idx = -(g + 1) is a gather block,
  // whose panel rows are B rows gather_rows[16g .. 16g + 15] (NULL: none)
  const int* gather_rows;
  // planned product (items NULL: item v is block row v / (ntiles * split)):
  // item v = items[v] = {block row, column tile, first block, end block}.
  // pair[v] = -1, or 128 * g + q for part q of split row (and tile) g, which
  // has parts[g] parts. Part 0 zeroes the C tile as soon as it takes the item
  // (its MMAs still running) and sets counters[2g]; every part waits for that
  // flag (bounded) and adds its tile into C with red.add; the last part to
  // count itself in counters[2g + 1] sets both back to zero.
  const int4* items;
  const int* pair;
  const int* parts;
  unsigned* counters;
  // e4m3: A's per-block scales (powers of two; each block's UE8M0 scale factor
  // is its exponent) and B's scale (applied in the epilogue)
  const float* scales;
  float b_scale;
  // stacked plan (stk > 1, fp16 / bf16, 64-row kernels): each 64-row block is
  // assembled in the stage from stk member blocks of mbR rows of A's own
  // values; smap holds, per stacked block and member, the source block or -1
  // (rows of zeros, read from row oob_row, past the end of A's tensor map)
  const int* smap;
  int stk, mbR, oob_row;
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* ptr) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ptr) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* ptr, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(ptr), "r"(v) : "memory");
}

// BR: block height (the UMMA N); NT: output columns per item; STAGES: ring
// depth in groups; ACC: TMEM accumulators per CTA (2 = one item's epilogue
// overlaps the next item's MMAs inside the CTA; 1 = half the TMEM, so two CTAs
// share an SM and overlap each other instead); G: blocks per group. A group is
// up to G consecutive stored blocks of one block row: one ring slot holds
// their A blocks (one TMA copy for a full group, the blocks are contiguous) and
// their G B panels, and one mbarrier pair tracks it. (An mbarrier wait in the
// thread that issues UMMAs costs ~200 cycles once UMMAs are in flight, so the
// MMA thread waits and commits once per group, not once per block.)
//
// E4M3 (MODE_E4M3) runs the same pipeline on the block-scaled MMA
// (kind::mxf8f6f4, K = 32, one UE8M0 scale factor per row and column for the
// 32-element K block). A block is 16 wide, so each block is one K = 32 MMA
// whose second K half is zero on the A side (the block descriptor's
// K-direction core-matrix stride points at a zeroed region after the group's
// blocks) and, on the panel side, reads the next 2 KB of the slot: the next
// 128-column slice, the next block's panel, or the slot's zero tail (a
// partial group's panels fill the slot's last slots, so its last block is
// followed by the tail too). A's per-block scale (a power of two) becomes the
// MMA's B-side scale factor: a 512-byte tile whose every 32-bit word holds the
// group's UE8M0 bytes (byte b for block b), written by one B issuer into the
// ring slot and moved to TMEM with one tcgen05.cp per group by each MMA
// issuer (into its own columns); the MMA of block b selects byte b with its
// scale-factor id. Every word is the same, so the factor does not depend on
// which TMEM lanes the MMA reads. The panel side's factor is a constant 1
// (0x7F), copied once per CTA and issuer. B's scale multiplies C
// in the epilogue.
template <int BR, int NT, int STAGES, int MODE, int ACC, int G>
struct TcCfg {
  static constexpr bool kSplit = MODE == MODE_SPLIT;
  static constexpr bool kE4 = MODE == MODE_E4M3;
  // a stacked plan's 64-row blocks are assembled from member blocks (fp16 / bf16)
  static constexpr bool kStackable = (MODE == MODE_F16 || MODE == MODE_BF16) && BR == 64;
  static constexpr int kParts = kSplit ? 2 : 1;
  static constexpr int kJ = NT / 128;                 // 128-column MMA slices per item
  // UMMA issuing threads: one thread's issue rate bounds the pipeline (a UMMA
  // takes the issuing thread ~74 cycles; doubling each block's UMMAs slowed
  // the headline plan by 17 %, while the same count at a quarter of the tensor
  // work saved 1-2 %), so two warps split each block's slices: disjoint
  // accumulators, the same sums. In e4m3 each issuer copies the scale factors
  // into its own TMEM columns, so every copy precedes the MMAs that read it in
  // one thread's issue order.
  static constexpr int kIssuers = kJ < 2 ? 1 : 2;
  static constexpr int kJPer = kJ / kIssuers;         // slices per issuer
  static constexpr int kBoxBytes = 16 * 128;          // 16 rows x 128 bytes: 64 fp16 or 128 e4m3 columns
  static constexpr int kBoxCols = kE4 ? 128 : 64;
  static constexpr int kPanelBytes = (NT / kBoxCols) * kBoxBytes;
  static constexpr int kSliceBytes = kPanelBytes / kJ;   // one 128-column slice of a panel
  static constexpr int kABytes = BR * (kE4 ? 16 : 32);   // bR rows x 16 elements
  static constexpr int kAPart = G * kABytes;          // one part (hi or lo) of a group's A blocks
  // fp16 / bf16 / split slot: [A (hi, lo) | B panels (hi, lo)]
  // e4m3 slot: [A blocks | zeros (one block) | scale tile | B panels | 2 KB zero tail]
  static constexpr int kAZeroOff = kAPart;
  static constexpr int kScaleOff = kAZeroOff + kABytes;
  static constexpr int kAStage = kE4 ? ((kScaleOff + 512 + 1023) / 1024) * 1024
                                     : ((kAPart * kParts + 1023) / 1024) * 1024;
  static constexpr int kTailOff = kAStage + G * kPanelBytes * kParts;
  static constexpr int kStage = kE4 ? ((kTailOff + 2048 + 1023) / 1024) * 1024 : kTailOff;
  // e4m3, after the ring: the panel-side scale tile (512 bytes of 0x7F)
  static constexpr int kExtra = kE4 ? 512 : 0;
  static constexpr int kAccCols = kJ * BR;            // TMEM columns of one accumulator
  // e4m3 scale factors in TMEM, per MMA issuer i: 4 columns for the panel
  // side (kSfaCol + 4 i), 4 per ring slot s (kSfbCol + 4 (i STAGES + s))
  static constexpr int kSfaCol = ACC * kAccCols;
  static constexpr int kSfbCol = kSfaCol + 4 * kIssuers;
  static constexpr int kUsedCols = kE4 ? kSfbCol + 4 * STAGES * kIssuers : ACC * kAccCols;
  static constexpr int kTmemCols = kUsedCols <= 32 ? 32 : kUsedCols <= 64 ? 64 : kUsedCols <= 128 ? 128
                                   : kUsedCols <= 256 ? 256 : 512;
  static constexpr size_t kSmem = 1024 + (size_t)STAGES * kStage + kExtra + 1024;
  static_assert(kUsedCols <= 512, "TMEM columns");
  static_assert(NT % 128 == 0, "NT");
  static_assert(G * BR <= 256 && 32 % G == 0, "a group is one TMA box and never straddles an index chunk");
  static_assert(!kE4 || G <= 4, "e4m3: one scale byte per block in a 32-bit word");
  // kind::f16 instruction descriptor: D f32, A/B f16 or bf16, A MN-major, B K-major,
  // N = BR, M = 128.
  static constexpr uint32_t kIdescF16 = (1u << 4) | ((MODE == MODE_BF16 ? 1u : 0u) << 7) |
                                        ((MODE == MODE_BF16 ? 1u : 0u) << 10) | (1u << 15) |
                                        ((uint32_t)(BR >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
  // kind::mxf8f6f4 block-scaled descriptor: A and B e4m3 (format 0), A MN-major,
  // B K-major, N = BR, UE8M0 scale factors, M = 128, scale-factor ids 0.
  static constexpr uint32_t kIdescE4 =
      (1u << 15) | ((uint32_t)(BR >> 3) << 17) | (1u << 23) | ((uint32_t)(128 >> 4) << 24);
  static constexpr uint32_t kIdesc = kE4 ? kIdescE4 : kIdescF16;
};

constexpr int kTcThreads = 352;   // 11 warps

template <int BR, int NT, int STAGES, int MODE, int ACC, int G>
__global__ void __launch_bounds__(kTcThreads, 2)
    k_bcsr_tc(const __grid_constant__ CUtensorMap tmA1, const __grid_constant__ CUtensorMap tmAg,
              const __grid_constant__ CUtensorMap tmAlo1, const __grid_constant__ CUtensorMap tmAlog,
              const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo,
              const TcParams p) {
  using Cfg = TcCfg<BR, NT, STAGES, MODE, ACC, G>;
  constexpr int kQ = 4;                       // item hand-off ring depth
  constexpr int kBIssuers = 4;
  constexpr int kScaleWriter = 3;             // e4m3: the B issuer that writes the scale tiles
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)STAGES * Cfg::kStage + Cfg::kExtra);
  // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], done, qfull[kQ], qempty[kQ];
  // then the TMEM address and the item ring
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES;
  const uint32_t tfull0 = empty0 + 8 * STAGES, tempty0 = tfull0 + 16, done_bar = tempty0 + 16;
  const uint32_t qfull0 = done_bar + 8, qempty0 = qfull0 + 8 * kQ;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5 + 2 * kQ);
  int* s_item = reinterpret_cast<int*>(tmem_slot + 1);      // kQ x {item, start, end, column tile}
  int* s_role = s_item + 4 * kQ;                            // a split row's role, set by the epilogue

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 32) {
    for (int s = 0; s < STAGES; ++s) {
      // the lead's arrive (it expects the whole group's bytes); e4m3 also B
      // issuer 0's, after it has written the group's scale tiles
      mbar_init(full0 + 8 * s, Cfg::kE4 ? 2 : 1);
      mbar_init(empty0 + 8 * s, Cfg::kIssuers);   // each MMA issuer's commit
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull0 + 8 * b, Cfg::kIssuers);
      mbar_init(tempty0 + 8 * b, 4);
    }
    mbar_init(done_bar, Cfg::kIssuers);
    for (int q = 0; q < kQ; ++q) {
      mbar_init(qfull0 + 8 * q, 1);
      mbar_init(qempty0 + 8 * q, Cfg::kIssuers + kBIssuers + 4);   // MMA issuers, B issuers, epilogue warps
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
  // A CTA's first item is blockIdx.x (the grid never exceeds the item count).
  // A plan's item list is the library's own, written when the plan was made,
  // so its first entry is read before the wait for the previous kernel in the
  // stream; everything the caller passes is read after it.
  int4 first = make_int4(0, 0, 0, 0);
  if (warp == 0 && lane == 0 && p.items) first = __ldg(p.items + blockIdx.x);
  if constexpr (Cfg::kE4) {
    // Zero each slot's A-side zero block and panel tail (never written by a
    // copy), fill the panel-side scale tile with UE8M0 1.0, and make the
    // stores visible to the tensor core's operand reads.
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    for (int i = threadIdx.x; i < STAGES * (Cfg::kABytes / 16); i += kTcThreads) {
      const int s = i / (Cfg::kABytes / 16), c = i % (Cfg::kABytes / 16);
      *reinterpret_cast<uint4*>(smem + (size_t)s * Cfg::kStage + Cfg::kAZeroOff + 16 * c) = z;
    }
    for (int i = threadIdx.x; i < STAGES * (2048 / 16); i += kTcThreads) {
      const int s = i / (2048 / 16), c = i % (2048 / 16);
      *reinterpret_cast<uint4*>(smem + (size_t)s * Cfg::kStage + Cfg::kTailOff + 16 * c) = z;
    }
    if (threadIdx.x < 32)
      *reinterpret_cast<uint4*>(smem + (size_t)STAGES * Cfg::kStage + 16 * threadIdx.x) =
          make_uint4(0x7F7F7F7Fu, 0x7F7F7F7Fu, 0x7F7F7F7Fu, 0x7F7F7F7Fu);
    fence_proxy_async_smem();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  grid_dep_launch_dependents();
  // The wait for the previous kernel on the stream (programmatic dependent
  // launch). With inputs_ready the caller promises that no kernel launched on
  // the stream since its last host synchronisation writes A or B, so the
  // warps that read only A and B or work in
  // shared memory and TMEM (lead, both MMA issuers, B issuers) start at once: a CTA copies
  // and multiplies its first item while the previous kernel finishes. The lead
  // waits before its first work-queue claim and the epilogue before it touches
  // C or a split row's counters, so the queue, the counters and C keep their
  // order with the previous kernel.
  const bool early = p.inputs_ready && (warp <= 3 || warp >= 8);
  if (!early) grid_dep_wait();
  bool dep_waited = !early;

  // Ring entry `it` of the item stream (bounded wait); *item < 0 ends the stream.
  auto read_item = [&](uint32_t it, int* item, int* start, int* end, unsigned code, int* tile = nullptr) -> bool {
    const uint32_t q = it % kQ;
    if (!mbar_wait(qfull0 + 8 * q, (it / kQ) & 1, p.timeout_ns)) {
      atomicOr(p.err, code);
      return false;
    }
    *item = s_item[4 * q];
    *start = s_item[4 * q + 1];
    *end = s_item[4 * q + 2];
    if (tile) *tile = s_item[4 * q + 3];
    mbar_arrive(qempty0 + 8 * q);
    return true;
  };
  const int bidx = warp == 2 ? 0 : warp == 3 ? 1 : warp == 8 ? 2 : warp == 9 ? 3 : -1;

  if (warp == 0) {
    // ------------------------------ lead producer ----------------------------------
    // Takes items (work queue or static stride), publishes them through the item
    // ring (-1 ends the stream), and for each group of the item's blocks claims
    // the ring slot, expects the group's bytes on its full barrier and copies the
    // A blocks. The B issuers copy the group's B panels into the same slot.
    if (lane == 0) {
      tma_prefetch_desc(&tmAg);
      tma_prefetch_desc(&tmA1);
      const uint64_t pol_a = l2_policy_evict_first();
      uint32_t gs = 0, it = 0;
      bool failed = false;
      // block range and column tile of an item: its block row's range, or one
      // of p.split slices of it (slice lengths a multiple of 4 blocks, so that
      // only a row's last slice can end in a partial group)
      auto range = [&](int v, int* s0, int* s1, int* tile) {
        if (v < 0) {
          *s0 = *s1 = *tile = 0;
          return;
        }
        if (p.items) {
          const int4 d = __ldg(p.items + v);
          *s0 = d.z;
          *s1 = d.w;
          *tile = d.y;
          return;
        }
        *tile = (v / p.split) % p.ntiles;
        const int row = v / (p.ntiles * p.split);
        int a = __ldg(p.row_ptr + row), b = __ldg(p.row_ptr + row + 1);
        if (p.split > 1) {
          const int k = v % p.split;
          const int chunk = (((b - a) + p.split - 1) / p.split + 3) & ~3;
          const int a2 = min(b, a + k * chunk);
          b = min(b, a2 + chunk);
          a = a2;
        }
        *s0 = a;
        *s1 = b;
      };
      // ring entry `e` := (v, s0, s1, tile); a wait for the slot that gives up ends the stream
      auto publish = [&](uint32_t e, int v, int s0, int s1, int tile) {
        const uint32_t q = e % kQ;
        if (e >= (uint32_t)kQ && !mbar_wait(qempty0 + 8 * q, ((e / kQ) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 4u);
          failed = true;
        }
        s_item[4 * q] = failed ? -1 : v;
        s_item[4 * q + 1] = s0;
        s_item[4 * q + 2] = s1;
        s_item[4 * q + 3] = tile;
        mbar_arrive(qfull0 + 8 * q);
      };
      // Items after the first: static striding (blockIdx.x + k * gridDim.x),
      // or tickets from the work queue offset by the grid size. A ticket is
      // taken late, when claim_ahead groups of the current item are left to
      // copy (< 0: as the item starts), so that a CTA running faster (lighter
      // items, or an SM it no longer shares) takes more of the items still
      // unclaimed; its atomic is issued one group before the result is used,
      // and the item goes into the ring at once. Either way every CTA takes
      // its items in increasing list order.
      const bool late = p.queue != nullptr && p.claim_ahead >= 0;
      auto ticket_item = [&](unsigned t) -> int {
        const unsigned v = t + gridDim.x;
        return v < (unsigned)p.n_items ? (int)v : -1;
      };
      int item = (int)blockIdx.x;
      int start = 0, end = 0, tile = 0;
      if (p.items) {
        start = first.z;
        end = first.w;
        tile = first.y;
      } else {
        range(item, &start, &end, &tile);
      }
      bool in_ring = false;
      for (;; ++it) {
        if (!in_ring) publish(it, item, start, end, tile);
        if (item < 0 || failed) break;
        int nitem = -2, nstart = 0, nend = 0, ntile = 0;
        bool claimed = false;
        unsigned ticket = 0;
        if (!late) {
          // the next item's indices load now and are used once this item is copied
          if (p.queue && !dep_waited) {
            grid_dep_wait();
            dep_waited = true;
          }
          nitem = p.queue ? ticket_item(atomicAdd(p.queue, 1u))
                          : (item + (int)gridDim.x < p.n_items ? item + (int)gridDim.x : -1);
          range(nitem, &nstart, &nend, &ntile);
        }
        const int ngroups = (end - start + G - 1) / G;
        if constexpr (MODE == MODE_F16 || MODE == MODE_BF16) {
          // A row's blocks are contiguous: one L2 prefetch of the whole item's A
          // takes its later groups' DRAM latency off their copies (measured
          // 1-2 % on back-to-back plans of the headline product; no effect on
          // e4m3 or on a launch timed alone)
          if (end > start && p.stk <= 1)
            tma_prefetch_l2(p.avals + (size_t)start * Cfg::kABytes, (uint32_t)((end - start) * Cfg::kABytes));
        }
        int gi = 0;
        for (int j0 = start; j0 < end; j0 += G, ++gs, ++gi) {
          if (late && nitem == -2) {
            if (claimed) {
              nitem = ticket_item(ticket);
              range(nitem, &nstart, &nend, &ntile);
              publish(it + 1, nitem, nstart, nend, ntile);
              if (failed) break;
            } else if (ngroups - gi <= p.claim_ahead + 1) {
              if (!dep_waited) {
                grid_dep_wait();
                dep_waited = true;
              }
              ticket = atomicAdd(p.queue, 1u);
              claimed = true;
            }
          }
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
          if constexpr (Cfg::kE4) {
            // unswizzled e4m3 blocks: the group's n blocks are contiguous in
            // memory and in the slot, one bulk copy
            tma_bulk_g2s(smem_u32(a_dst), p.avals + (size_t)j0 * Cfg::kABytes, (uint32_t)(n * Cfg::kABytes), fb,
                         pol_a);
          } else if (Cfg::kStackable && p.stk > 1) {
            // a stacked block's members are copied by the B issuers
          } else if (n == G) {
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
        in_ring = late && nitem != -2;
        if (nitem == -2) {   // late claim not made or not used yet (short item)
          if (!claimed) {
            if (!dep_waited) {
              grid_dep_wait();
              dep_waited = true;
            }
            ticket = atomicAdd(p.queue, 1u);
          }
          nitem = ticket_item(ticket);
          range(nitem, &nstart, &nend, &ntile);
        }
        item = nitem;
        start = nstart;
        end = nend;
        tile = ntile;
      }
      // the last CTA to finish resets the queue for the next launch
      if (p.queue) {
        if (!dep_waited) grid_dep_wait();
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
    // Issuer k copies the B panel of block b of each group with b % 4 == k into
    // the group's slot (a TMA copy holds its issuing thread for ~200 ns, so four
    // threads share the panels). Its lanes stage column indices 32 at a time,
    // prefetching the next chunk while lane 0 issues.
    if (lane == 0) tma_prefetch_desc(&tmB);
    const uint64_t pol_b = l2_policy_evict_last();
    uint32_t gs = 0;
    int failed = 0;
    for (uint32_t it = 0; !failed; ++it) {
      int item = -1, start = 0, end = 0, nt = 0, ok = 1;
      if (lane == 0) ok = read_item(it, &item, &start, &end, 4u, &nt) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      item = __shfl_sync(0xffffffffu, item, 0);
      start = __shfl_sync(0xffffffffu, start, 0);
      end = __shfl_sync(0xffffffffu, end, 0);
      nt = __shfl_sync(0xffffffffu, nt, 0);
      if (!ok || item < 0) break;
      // One pass over the item's blocks. A stacked plan also copies, per
      // stacked block, its member blocks from A's values into the block's A
      // slot; the two cases are separate instantiations, so the plain path
      // carries none of the member work.
      auto issue_item = [&](auto stacked_tag) {
        constexpr bool kStacked = decltype(stacked_tag)::value;
        // member blocks take the lead's policy for A
        const uint64_t pol_a = kStacked ? l2_policy_evict_first() : 0ull;
        int mycol = lane < end - start ? __ldg(p.col_idx + start + lane) : 0;
        // a stacked plan: each lane also stages the member source blocks of its
        // stacked block (stk of them, -1 where the member row has no block)
        const int stk = kStacked ? p.stk : 1;
        auto load_members = [&](int j, int (&mm)[4]) {
#pragma unroll
          for (int t = 0; t < 4; ++t) mm[t] = (t < stk && j < end) ? __ldg(p.smap + (long long)j * stk + t) : -1;
        };
        int mym[4] = {-1, -1, -1, -1};
        if constexpr (kStacked) load_members(start + lane, mym);
        // e4m3, the scale writer (issuer 3): the blocks' scales, staged like the column indices
        float mysc = 1.f;
        if constexpr (Cfg::kE4) {
          if (bidx == kScaleWriter) mysc = lane < end - start ? __ldg(p.scales + start + lane) : 1.f;
        }
        for (int base = start; base < end && !failed; base += 32) {
          const int cnt = min(32, end - base);
          const int cur = mycol;
          [[maybe_unused]] const float cursc = mysc;
          int curm[4] = {mym[0], mym[1], mym[2], mym[3]};
          if constexpr (kStacked)
            if (base + 32 < end) load_members(base + 32 + lane, mym);
          if (base + 32 < end) mycol = lane < end - base - 32 ? __ldg(p.col_idx + base + 32 + lane) : 0;
          if constexpr (Cfg::kE4) {
            if (bidx == kScaleWriter && base + 32 < end)
              mysc = lane < end - base - 32 ? __ldg(p.scales + base + 32 + lane) : 1.f;
          }
          for (int i0 = 0; i0 < cnt; i0 += G, ++gs) {
            const int n = min(G, cnt - i0);
            const int s = (int)(gs % STAGES);
            // Wait for the slot only in groups this issuer copies into: such a
            // group cannot be released without its bytes, so the slot's empty
            // barrier is at most one phase ahead. (An issuer that also waited in
            // groups it has no block in could fall two phases behind and miss a
            // parity flip.) Issuer 0 copies into every group, and so does the
            // e4m3 scale writer (its arrival is part of every group's full barrier).
            // The parity test is only valid when group gs - 2 * STAGES has been
            // consumed (otherwise a stale parity reads as free). Consumption is in
            // order, so the wait in an issuer's previous group covers it as long as
            // that group is at most STAGES groups back: issuers skip only an item's
            // last, partial group, and the lead publishes an item once the group
            // 2 * STAGES before its first has been consumed (claim_ahead = STAGES - 1).
            // (Rotating the block-to-issuer map over groups of fewer than four
            // blocks breaks this and was measured to corrupt a slot.)
            const bool writes = bidx < n || (Cfg::kE4 && bidx == kScaleWriter);
            int bad = 0;
            if (lane == 0 && writes && gs >= (uint32_t)STAGES &&
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
              if constexpr (!Cfg::kSplit && !Cfg::kE4 && !kStacked) {
                if (col < 0 && p.gather_rows) {
                  // Gather block: its panel is 16 arbitrary B rows. Lane L < 4 * (NT / 64)
                  // copies rows 4q .. 4q + 3 (q = L % 4) of 64-column box L / 4 with one
                  // tile::gather4 (tmBlo is then the one-row-box view of B), into the
                  // box's rows 4q .. 4q + 3: the image of a 16-row box copy. Padding
                  // rows index K, past the end of B, and read zeros.
                  const long long g = -(long long)col - 1;
                  const int kk = lane < 16 ? __ldg(p.gather_rows + 16 * g + lane) : 0;
                  const int q = lane & 3;
                  const int y0 = __shfl_sync(0xffffffffu, kk, 4 * q);
                  const int y1 = __shfl_sync(0xffffffffu, kk, 4 * q + 1);
                  const int y2 = __shfl_sync(0xffffffffu, kk, 4 * q + 2);
                  const int y3 = __shfl_sync(0xffffffffu, kk, 4 * q + 3);
                  if (lane < 4 * (NT / 64)) {
                    const int bx = lane >> 2;
                    tma_gather4_g2s(smem_u32(b_dst0 + (size_t)b * Cfg::kPanelBytes + bx * Cfg::kBoxBytes + q * 512),
                                    &tmBlo, nt * NT + bx * 64, y0, y1, y2, y3, full0 + 8 * s, pol_b);
                  }
                  continue;
                }
              }
              if (lane == 0) {
                const uint32_t fb = full0 + 8 * s;
                if constexpr (kStacked) {
                  // the stacked 64-row block: member t's rows at t * mbR, from
                  // its source block, or a box past the end of A (zeros)
                  uint8_t* a_dst = smem + (size_t)s * Cfg::kStage + (size_t)b * Cfg::kABytes;
#pragma unroll
                  for (int t = 0; t < 4; ++t)
                    if (t < stk)
                      tma_tile_2d_g2s(smem_u32(a_dst + t * p.mbR * 32), &tmA1, 0,
                                      src[t] >= 0 ? src[t] * p.mbR : p.oob_row, fb, pol_a);
                }
                // e4m3: a partial group's panels take the slot's last slots
                const int slot = Cfg::kE4 ? G - n + b : b;
                uint8_t* b_dst = b_dst0 + (size_t)slot * Cfg::kPanelBytes * Cfg::kParts;
                const int y = col * 16;
                if (p.panel3d) {
                  tma_tile_3d_g2s(smem_u32(b_dst), &tmB, 0, y, nt * (NT / Cfg::kBoxCols), fb, pol_b);
                  if (Cfg::kSplit)
                    tma_tile_3d_g2s(smem_u32(b_dst + Cfg::kPanelBytes), &tmBlo, 0, y, nt * (NT / 64), fb, pol_b);
                } else {
#pragma unroll
                  for (int bx = 0; bx < NT / Cfg::kBoxCols; ++bx) {
                    tma_tile_2d_g2s(smem_u32(b_dst + bx * Cfg::kBoxBytes), &tmB, nt * NT + bx * Cfg::kBoxCols, y, fb,
                                    pol_b);
                    if (Cfg::kSplit)
                      tma_tile_2d_g2s(smem_u32(b_dst + Cfg::kPanelBytes + bx * Cfg::kBoxBytes), &tmBlo,
                                      nt * NT + bx * 64, y, fb, pol_b);
                  }
                }
              }
            }
            if constexpr (Cfg::kE4) {
              if (bidx == kScaleWriter) {
                // After its own copies are in flight: the group's 512-byte scale
                // tile, every 32-bit word holding byte b = block b's scale in
                // UE8M0, the exponent field of a power-of-two fp32 (bit 64 of
                // the error word flags a scale that is not one); then the proxy
                // fence that makes it visible to tcgen05.cp, and the arrival the
                // group's full barrier waits for.
                uint32_t w = 0;
                for (int b = 0; b < n; ++b) {
                  const uint32_t bits = __float_as_uint(__shfl_sync(0xffffffffu, cursc, i0 + b));
                  const uint32_t e = (bits >> 23) & 0xFFu;
                  if (lane == 0 && ((bits & 0x807FFFFFu) != 0u || e == 0u || e == 0xFFu)) atomicOr(p.err, 64u);
                  w |= e << (8 * b);
                }
                *reinterpret_cast<uint4*>(smem + (size_t)s * Cfg::kStage + Cfg::kScaleOff + 16 * lane) =
                    make_uint4(w, w, w, w);
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(full0 + 8 * s);
              }
            }
          }
        }
      };
      if constexpr (Cfg::kStackable) {
        if (p.stk > 1) {
          issue_item(std::true_type{});
          continue;
        }
      }
      issue_item(std::false_type{});
    }
  } else if (warp == 1 || (Cfg::kIssuers == 2 && warp == 10)) {
    // ------------------------------ MMA issuers ----------------------------------
    // Issuer i takes 128-column slices [i * kJPer, (i + 1) * kJPer) of every
    // block; each commits its own MMAs to the slot, accumulator and done
    // barriers, which expect one commit per issuer.
    if (lane == 0) {
      const int mi = warp == 1 ? 0 : 1;
      const int jb = mi * Cfg::kJPer;
      const uint32_t sfa = tmem + Cfg::kSfaCol + 4 * mi;
      uint32_t gs = 0, it = 0;
      bool failed = false;
      if constexpr (Cfg::kE4)   // the panel side's scale factors: 1.0 for every row
        tmem_cp_32x128b_x4(sfa, smem_desc(smem_u32(smem + (size_t)STAGES * Cfg::kStage), 128, 128, kLayoutNone));
      for (;; ++it) {
        int item, start, end;
        if (!read_item(it, &item, &start, &end, 8u) || item < 0) break;
        const uint32_t acc = it % ACC;
        if (it >= (uint32_t)ACC && !mbar_wait(tempty0 + 8 * acc, ((it / ACC) + 1) & 1, p.timeout_ns)) {
          atomicOr(p.err, 8u);
          break;
        }
        tc_fence_after();
        const uint32_t d0 = tmem + acc * Cfg::kAccCols;
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
          // e4m3: the group's scale factors into the slot's TMEM columns, ahead of its MMAs
          const uint32_t sfb = tmem + Cfg::kSfbCol + (uint32_t)((mi * STAGES + s) * 4);
          if constexpr (Cfg::kE4)
            tmem_cp_32x128b_x4(sfb, smem_desc(a_slot + Cfg::kScaleOff, 128, 128, kLayoutNone));
          for (int b = 0; b < n; ++b) {
            const uint32_t b_addr = b_slot + (Cfg::kE4 ? G - n + b : b) * Cfg::kPanelBytes * Cfg::kParts;
            const uint32_t accum = (j0 + b != start) ? 1u : 0u;
            if constexpr (Cfg::kE4) {
              // one K = 32 MMA per slice: K 0..15 the block (K-major, no
              // swizzle, 8-row core matrices 128 bytes apart), K 16..31 the
              // slot's zero block; scale-factor id b picks the block's byte
              const uint32_t blk = a_slot + b * Cfg::kABytes;
              const uint64_t blk_d = smem_desc(blk, a_slot + Cfg::kAZeroOff - blk, 128, kLayoutNone);
#pragma unroll
              for (int jj = 0; jj < Cfg::kJPer; ++jj) {
                const int j = jb + jj;
                const uint64_t pan = smem_desc(b_addr + j * Cfg::kSliceBytes, 1024, 1024, kLayoutSW128);
                umma_mxf8_scaled(d0 + j * BR, pan, blk_d, Cfg::kIdesc | ((uint32_t)b << 4), sfa, sfb, accum);
              }
              continue;
            }
            const uint64_t blk_hi = smem_desc(a_slot + b * Cfg::kABytes, 16, 256, kLayoutSW32);
#pragma unroll
            for (int jj = 0; jj < Cfg::kJPer; ++jj) {
              const int j = jb + jj;
              const uint64_t pan_hi = smem_desc(b_addr + j * 2 * Cfg::kBoxBytes, 2048, 1024, kLayoutSW128);
              umma_f16(d0 + j * BR, pan_hi, blk_hi, Cfg::kIdesc, accum);
              if constexpr (Cfg::kSplit) {
                const uint64_t pan_lo =
                    smem_desc(b_addr + Cfg::kPanelBytes + j * 2 * Cfg::kBoxBytes, 2048, 1024, kLayoutSW128);
                const uint64_t blk_lo =
                    smem_desc(a_slot + Cfg::kAPart + b * Cfg::kABytes, 16, 256, kLayoutSW32);
                umma_f16(d0 + j * BR, pan_lo, blk_hi, Cfg::kIdesc, 1u);
                umma_f16(d0 + j * BR, pan_hi, blk_lo, Cfg::kIdesc, 1u);
              }
            }
          }
          umma_commit(empty0 + 8 * s);   // frees the group's slot once these MMAs have read it
        }
        if (failed) break;
        umma_commit(tfull0 + 8 * acc);   // accumulator ready (immediately, for an empty row)
      }
      // every MMA the issuers issued has completed before TMEM is released
      umma_commit(done_bar);
      if (!mbar_wait(done_bar, 0, p.timeout_ns)) atomicOr(p.err, 8u);
    }
    __syncwarp();
  } else if (warp >= 4 && warp < 8) {
    // ------------------------------ epilogue (warps 4-7) ---------------------------
    const int q4 = warp & 3;                // TMEM lane quarter this warp may access
    const bool hybrid = p.csr_row_ptr != nullptr;
    const bool planned = p.pair != nullptr;
    for (uint32_t it = 0;; ++it) {
      int item = -1, start = 0, end = 0, ok = 1;
      if (lane == 0) ok = read_item(it, &item, &start, &end, 16u) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      item = __shfl_sync(0xffffffffu, item, 0);
      const bool empty = __shfl_sync(0xffffffffu, start == end ? 1 : 0, 0) != 0;
      bool leave = !ok || item < 0;
      int br = 0, nt = 0, grp = -1, part = 0;
      if (!leave) {
        if (p.items) {
          const int4 d = __ldg(p.items + item);
          br = d.x;
          nt = d.y;
        } else {
          br = item / (p.ntiles * p.split);
          nt = (item / p.split) % p.ntiles;
        }
        if (planned) {
          const int code = __ldg(p.pair + item);
          if (code >= 0) {
            grp = code >> 7;
            part = code & 127;
          }
        }
      }
      const long long row0 = (long long)br * BR;
      // The hybrid pass and the split-row protocol synchronise the four
      // epilogue warps, so they agree on leaving (a reduction over the same
      // named barrier) and no warp is left waiting for one that has gone.
      if (planned) {
        if (bar_red_or(1, 128, leave)) break;
        if (grp >= 0 && part == 0) {
          // part 0 of a split row: zero its C tile while the MMAs run
          const int n0 = nt * NT, n1 = min(nt * NT + NT, p.N);
          for (int r = q4; r < BR; r += 4) {
            float* crow = p.C + (row0 + r) * p.ldc;
            for (int n = n0 + lane * 4; n < n1; n += 128) __stcg(reinterpret_cast<float4*>(crow + n), make_float4(0.f, 0.f, 0.f, 0.f));
          }
          __threadfence();
          bar_sync_named(1, 128);
          if (warp == 4 && lane == 0) st_release_gpu(p.counters + 2 * grp, 1u);
        }
      }
      if (!leave && !mbar_wait(tfull0 + 8 * (it % ACC), (it / ACC) & 1, p.timeout_ns)) {
        if (lane == 0) atomicOr(p.err, 16u);
        leave = true;
      }
      if ((hybrid || planned) ? bar_red_or(1, 128, leave) : leave) break;
      tc_fence_after();
      const uint32_t acc = (it % ACC);
      // a part of a split row adds into C once part 0 has zeroed it (role 2);
      // role 3: the wait gave up (error word set), nothing is added
      int role = 0;
      if (grp >= 0) {
        if (warp == 4 && lane == 0) {
          int r = 2;
          const uint64_t t0 = global_timer_ns();
          while (ld_acquire_gpu(p.counters + 2 * grp) == 0) {
            if (global_timer_ns() - t0 > p.timeout_ns) {
              atomicOr(p.err, 32u);
              r = 3;
              break;
            }
            __nanosleep(64);
          }
          *s_role = r;
        }
        bar_sync_named(1, 128);
        role = *reinterpret_cast<volatile int*>(s_role);
        __threadfence();
      }
      if (role != 3) {
#pragma unroll 1
        for (int j = 0; j < Cfg::kJ; ++j) {
          const int n = nt * NT + j * 128 + q4 * 32 + lane;
          float* cptr = p.C + row0 * p.ldc + n;
          const uint32_t taddr = tmem + ((uint32_t)(q4 * 32) << 16) + acc * Cfg::kAccCols + j * BR;
#pragma unroll
          for (int c0 = 0; c0 < BR; c0 += 16) {
            float v[16];
            if (!empty) {
              tmem_ld16(taddr + c0, v);
              if constexpr (Cfg::kE4) {
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] *= p.b_scale;
              }
            } else {
#pragma unroll
              for (int i = 0; i < 16; ++i) v[i] = 0.f;
            }
            if (n < p.N) {
              if (hybrid) {
                // read back by the CSR pass below: keep the lines in L2
#pragma unroll
                for (int i = 0; i < 16; ++i) cptr[(long long)(c0 + i) * p.ldc] = v[i];
              } else if (role == 2 || (p.split > 1 && !empty)) {
#pragma unroll
                for (int i = 0; i < 16; ++i) red_add_f32(cptr + (long long)(c0 + i) * p.ldc, v[i]);
              } else if (p.split == 1) {
#pragma unroll
                for (int i = 0; i < 16; ++i) __stcs(cptr + (long long)(c0 + i) * p.ldc, v[i]);
              }
            }
          }
        }
      }
      if (grp >= 0) {
        // count this part in; the last one resets the pair's counters
        __threadfence();
        bar_sync_named(1, 128);
        if (warp == 4 && lane == 0 && atomicAdd(p.counters + 2 * grp + 1, 1u) == (unsigned)__ldg(p.parts + grp) - 1u) {
          p.counters[2 * grp] = 0u;
          p.counters[2 * grp + 1] = 0u;
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty0 + 8 * acc);
      if (hybrid) {
        // The accumulator is free for the next item's MMAs; the CSR part of
        // this tile's rows is added to C in place. Each CTA owns its C tile
        // (no split-K here), and the named barrier orders the four warps'
        // stores above before any lane reads them back.
        bar_sync_named(1, 128);
        csr_tile_pass(p.csr_row_ptr, p.csr_col_idx, p.csr_vals, p.Bh, p.ldb, p.C, p.ldc, row0, BR,
                      nt * NT, min(nt * NT + NT, p.N), q4, lane);
      }
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
                      const CUtensorMap, const CUtensorMap, const TcParams);
struct TcEntry {
  int br, mode, nt, stages, acc, group;
  TcFn fn;
  size_t smem;
  int tmem_cols;
};
#define SPMM_TC_ENTRY(BR, NT, ST, MODE, ACC, G)                                            \
  TcEntry{BR, MODE, NT, ST, ACC, G, &k_bcsr_tc<BR, NT, ST, MODE, ACC, G>,                  \
          TcCfg<BR, NT, ST, MODE, ACC, G>::kSmem, TcCfg<BR, NT, ST, MODE, ACC, G>::kTmemCols}

// Instantiated (block height, column tile, ring depth in groups, accumulators,
// group size) per type.
// The first entry of a (block height, column tile) pair is its default. For
// 64-row blocks and 256 columns that is a ring of five 2-block groups (2 x 103
// KB of shared memory per SM): the pipeline is bound by the latency of its
// copies, and the fifth group measured ~2 % faster than four on the headline
// product.
#define SPMM_TC_SHAPES(MODE)                                                                         \
  SPMM_TC_ENTRY(64, 256, 5, MODE, 2, 2), SPMM_TC_ENTRY(64, 256, 4, MODE, 2, 2),                     \
      SPMM_TC_ENTRY(64, 256, 2, MODE, 2, 4),                                                        \
      SPMM_TC_ENTRY(64, 512, 3, MODE, 1, 2), SPMM_TC_ENTRY(64, 512, 3, MODE, 2, 4),                 \
      SPMM_TC_ENTRY(64, 128, 4, MODE, 2, 4), SPMM_TC_ENTRY(32, 256, 3, MODE, 2, 4),                 \
      SPMM_TC_ENTRY(32, 512, 3, MODE, 1, 2), SPMM_TC_ENTRY(16, 256, 3, MODE, 2, 4),                 \
      SPMM_TC_ENTRY(16, 512, 3, MODE, 1, 2)

const TcEntry kTcEntries[] = {
    SPMM_TC_SHAPES(MODE_F16),
    SPMM_TC_SHAPES(MODE_BF16),
    SPMM_TC_ENTRY(64, 256, 2, MODE_SPLIT, 2, 2),
    SPMM_TC_ENTRY(64, 128, 3, MODE_SPLIT, 2, 2),
    SPMM_TC_ENTRY(64, 512, 2, MODE_SPLIT, 1, 1),
    // e4m3: TMEM holds the accumulators and the scale factors (4 columns per
    // block of the ring), so the 512-column tile and two 256-column
    // accumulators run one CTA per SM
    SPMM_TC_ENTRY(64, 256, 7, MODE_E4M3, 1, 2), SPMM_TC_ENTRY(64, 512, 9, MODE_E4M3, 1, 2),
    SPMM_TC_ENTRY(64, 256, 8, MODE_E4M3, 2, 2), SPMM_TC_ENTRY(64, 128, 8, MODE_E4M3, 2, 2),
    SPMM_TC_ENTRY(64, 256, 4, MODE_E4M3, 1, 4), SPMM_TC_ENTRY(64, 512, 4, MODE_E4M3, 1, 4),
    SPMM_TC_ENTRY(32, 256, 4, MODE_E4M3, 1, 4), SPMM_TC_ENTRY(16, 256, 4, MODE_E4M3, 1, 4),
    SPMM_TC_ENTRY(16, 256, 3, MODE_E4M3, 2, 4),
};

int tc_mode(spmm_dtype d) {
  return d == SPMM_F16 ? MODE_F16 : d == SPMM_BF16 ? MODE_BF16 : d == SPMM_F16_SPLIT ? MODE_SPLIT
         : d == SPMM_E4M3 ? MODE_E4M3 : -1;
}

// The instantiation a request runs on (NULL if none): column tile (default 128
// for 64-row blocks and N <= 128, else 256), then the first entry matching the
// requested depth and accumulator count.
const TcEntry* find_tc(int bR, int mode, int N, const spmm_config& cfg, int* nt_out) {
  int nt = cfg.n_tile;
  if (nt <= 0) nt = (N <= 128 && bR == 64) ? 128 : 256;
  if (nt < 256 && bR != 64) nt = 256;
  *nt_out = nt;
  for (const TcEntry& c : kTcEntries) {
    if (c.br != bR || c.mode != mode || c.nt != nt) continue;
    if (cfg.stages > 0 && c.stages != cfg.stages) continue;
    if (cfg.acc_buffers > 0 && c.acc != cfg.acc_buffers) continue;
    return &c;
  }
  return nullptr;
}

}  // namespace

bool tc_supported(int bR, spmm_dtype dtype, int N, const spmm_config& cfg) {
  const int mode = tc_mode(dtype);
  int nt = 0;
  // a requested column tile must be the one that runs (find_tc widens 128 to 256 for 16- and 32-row blocks)
  return mode >= 0 && cfg.split_k <= 16 && find_tc(bR, mode, N, cfg, &nt) != nullptr &&
         (cfg.n_tile <= 0 || nt == cfg.n_tile);
}

bool tc_geometry(int bR, spmm_dtype dtype, int N, const spmm_config& cfg, int* nt, int* ctas_per_sm) {
  const int mode = tc_mode(dtype);
  if (mode < 0) return false;
  const TcEntry* e = find_tc(bR, mode, N, cfg, nt);
  if (!e) return false;
  const int tmem_fit = 512 / e->tmem_cols;
  const int smem_fit = smem_per_sm() / (int)(e->smem + 1024);
  int per_sm = std::min(2, std::min(tmem_fit, smem_fit));
  if (cfg.ctas_per_sm > 0 && cfg.ctas_per_sm < per_sm) per_sm = cfg.ctas_per_sm;
  *ctas_per_sm = per_sm < 1 ? 1 : per_sm;
  return true;
}

spmm_status launch_tc(const LaunchRequest& r) {
  const spmm_bcsr_desc& A = *r.A;
  const spmm_dense_desc& B = *r.B;
  const int mode = tc_mode(A.dtype);
  if (mode < 0) return fail(SPMM_ERR_UNSUPPORTED, "tcgen05 pipeline: fp16, bf16, split fp16 and e4m3 only");
  const bool e4 = mode == MODE_E4M3;
  if (e4 && (r.csr || r.gather_rows))
    return fail(SPMM_ERR_UNSUPPORTED, "the hybrid product and gather blocks run in fp16 / bf16");
  if (e4 && !A.scales) return fail(SPMM_ERR_INVALID_ARG, "E4M3 needs per-block scales");
  int nt = 0;
  const TcEntry* e = find_tc(A.bR, mode, r.N, r.cfg, &nt);
  if (!e)
    return fail(SPMM_ERR_UNSUPPORTED, "no tcgen05 kernel for bR=" + std::to_string(A.bR) +
                                          " n_tile=" + std::to_string(nt));
  // A's values viewed as a [rows x 16] fp16 tensor; rows bounded by the densest
  // possible matrix (only coordinates of stored blocks are ever requested: a
  // group copy is issued only for kGroup consecutive blocks of one block row).
  unsigned long long rows_bound =
      std::max<unsigned long long>((unsigned long long)(A.M / A.bR) * (A.K / 16) * A.bR, 256ull);
  if (r.gather_rows)   // gather blocks come on top of at most K / 16 stored blocks per row
    rows_bound = std::max<unsigned long long>(rows_bound, (unsigned long long)r.total_blocks * A.bR);
  const bool stacked = r.stack > 1;
  // (a stacked run also names row rows_bound, the first past the end, as the source of its zero members)
  if (rows_bound >= (1ull << 31) - (stacked ? 64 : 0))
    return fail(SPMM_ERR_UNSUPPORTED, "A too large for the tcgen05 pipeline");
  if (stacked && (A.bR != 64 || (mode != MODE_F16 && mode != MODE_BF16) || r.csr || r.gather_rows || !r.stack_map ||
                  (r.member_bR != 16 && r.member_bR != 32) || r.stack * r.member_bR != 64))
    return fail(SPMM_ERR_UNSUPPORTED, "a stacked run takes 16- or 32-row fp16 / bf16 blocks on the 64-row pipeline");
  CUtensorMap tmA1, tmAg, tmAlo1, tmAlog, tmB, tmBlo;
  const void* vals = A.vals ? A.vals : B.data;   // no stored blocks: never dereferenced
  // A's values as a [rows x 16] matrix: 16-bit with 32-byte swizzle (the UMMA
  // K-major SW32 layout), or e4m3 bytes unswizzled (K-major, 8 x 16-byte core
  // matrices, contiguous per block)
  const CUtensorMapDataType adt = e4 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
  const CUtensorMapSwizzle aswz = e4 ? CU_TENSOR_MAP_SWIZZLE_NONE : CU_TENSOR_MAP_SWIZZLE_32B;
  const uint64_t arow = e4 ? 16 : 32;
  // (a stacked run: A.vals holds the member blocks, bR = member_bR rows each,
  // and the same rows bound: (M / bR) * (K / 16) * bR rows for any bR)
  spmm_status st = encode_tile_map_2d(&tmA1, adt, vals, 16, rows_bound, arow, 16,
                                      (uint32_t)(stacked ? r.member_bR : A.bR), aswz);
  if (st != SPMM_OK) return st;
  st = encode_tile_map_2d(&tmAg, adt, vals, 16, rows_bound, arow, 16, (uint32_t)(e->group * A.bR), aswz);
  if (st != SPMM_OK) return st;
  // B panels: one 3-D copy per panel when N is a multiple of the 128-byte box
  // width (64 16-bit or 128 e4m3 columns), else one 2-D copy per box.
  const int esz = e4 ? 1 : 2, box_cols = 128 / esz;
  int panel3d = (r.N % box_cols == 0) ? 1 : 0;
  if (panel3d && encode_panel_map_3d(&tmB, B.data, (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * esz,
                                     (uint32_t)(nt / box_cols), esz) != SPMM_OK)
    panel3d = 0;
  if (!panel3d) {
    st = encode_tile_map_2d(&tmB, e4 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, B.data,
                            (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * esz, (uint32_t)box_cols, 16,
                            CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  }
  tmAlo1 = tmA1;
  tmAlog = tmAg;
  tmBlo = tmB;
  if (r.gather_rows) {
    // gather blocks: tmBlo becomes B viewed with a one-row box, the form tile::gather4 copies
    if (mode == MODE_SPLIT) return fail(SPMM_ERR_UNSUPPORTED, "gather blocks run in fp16 or bf16");
    st = encode_tile_map_2d(&tmBlo, CU_TENSOR_MAP_DATA_TYPE_UINT16, B.data, (uint64_t)r.N, (uint64_t)A.K,
                            (uint64_t)B.ldb * 2, 64, 1, CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  }
  if (mode == MODE_SPLIT) {
    const void* lo = A.vals_lo ? A.vals_lo : B.data_lo;
    st = encode_tile_map_2d(&tmAlo1, CU_TENSOR_MAP_DATA_TYPE_UINT16, lo, 16, rows_bound, 32, 16,
                            (uint32_t)A.bR, CU_TENSOR_MAP_SWIZZLE_32B);
    if (st != SPMM_OK) return st;
    st = encode_tile_map_2d(&tmAlog, CU_TENSOR_MAP_DATA_TYPE_UINT16, lo, 16, rows_bound, 32, 16,
                            (uint32_t)(e->group * A.bR), CU_TENSOR_MAP_SWIZZLE_32B);
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
  p.split = r.cfg.split_k > 1 ? r.cfg.split_k : 1;
  if (p.split > 16) return fail(SPMM_ERR_INVALID_ARG, "split_k must be at most 16");
  const long long n_items = (long long)(A.M / A.bR) * p.ntiles * p.split;
  if (n_items >= (1ll << 30)) return fail(SPMM_ERR_UNSUPPORTED, "too many work items");
  p.n_items = (int)n_items;
  p.timeout_ns = wait_limit_ns();
  p.err = r.err_word ? r.err_word : device_error_word();
  p.panel3d = panel3d;
  // items: static stride by default, or a work queue on request
  p.queue = r.queue ? r.queue : (r.cfg.schedule >= 1 ? work_queue_slot() : nullptr);
  p.claim_ahead = e->stages - 1;
  p.inputs_ready = r.inputs_ready ? 1 : 0;
  p.csr_row_ptr = r.csr ? r.csr->row_ptr : nullptr;
  p.csr_col_idx = r.csr ? r.csr->col_idx : nullptr;
  p.csr_vals = r.csr ? static_cast<const __half*>(r.csr->vals) : nullptr;
  p.Bh = static_cast<const __half*>(B.data);
  p.ldb = B.ldb;
  p.gather_rows = r.gather_rows;
  p.items = r.items;
  p.pair = r.pair;
  p.parts = r.parts;
  p.counters = r.counters;
  p.scales = A.scales;
  p.avals = static_cast<const uint8_t*>(A.vals);
  p.b_scale = e4 ? B.scale : 1.0f;
  p.smap = stacked ? r.stack_map : nullptr;
  p.stk = stacked ? r.stack : 1;
  p.mbR = stacked ? r.member_bR : 0;
  p.oob_row = (int)rows_bound;
  if (r.items) {
    if (p.split > 1 || r.csr || r.gather_rows || (p.queue && !r.queue))
      return fail(SPMM_ERR_UNSUPPORTED, "a planned product runs without split-K, CSR part or shared work queue");
    p.n_items = r.plan_items;
  }
  if (r.csr && (p.split > 1 || mode != MODE_F16))
    return fail(SPMM_ERR_UNSUPPORTED, "the hybrid product runs in fp16 without split-K");
  if (!p.err) return fail(SPMM_ERR_CUDA, "could not set up the device error word");
  if (p.n_items == 0) return SPMM_OK;
  if (p.split > 1)
    SPMM_CUDA_TRY(cudaMemset2DAsync(r.C, (size_t)r.ldc * 4, 0, (size_t)r.N * 4, A.M, r.stream));
  SPMM_CUDA_TRY(ensure_smem_attr(reinterpret_cast<const void*>(e->fn), (int)e->smem));
  // CTAs per SM from the real limits: TMEM columns (512 per SM), shared memory
  // per SM, and the two CTAs the launch bounds budget registers for. (The
  // runtime's occupancy query reports one CTA per SM for this kernel, while two
  // run side by side.)
  const int smem_sm = smem_per_sm();
  const int tmem_fit = 512 / e->tmem_cols;
  const int smem_fit = smem_sm / (int)(e->smem + 1024);
  int per_sm = std::min(2, std::min(tmem_fit, smem_fit));
  if (r.cfg.ctas_per_sm > 0 && r.cfg.ctas_per_sm < per_sm) per_sm = r.cfg.ctas_per_sm;
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)sm_count() * per_sm;
  if (grid > p.n_items) grid = p.n_items;
  if (std::getenv("SPMM_DEBUG"))
    std::fprintf(stderr,
                 "[spmm] tcgen05 bR=%d nt=%d stages=%d acc=%d group=%d smem=%zu tmem=%d per_sm=%d grid=%lld "
                 "items=%d panel3d=%d queue=%d claim_ahead=%d inputs_ready=%d split=%d\n",
                 A.bR, nt, e->stages, e->acc, e->group, e->smem, e->tmem_cols, per_sm, grid, p.n_items, panel3d,
                 p.queue != nullptr, p.claim_ahead, p.inputs_ready, p.split);
  SPMM_CUDA_TRY(launch_kernel(e->fn, dim3((unsigned)grid), dim3(kTcThreads), e->smem, r.stream, tmA1, tmAg, tmAlo1,
                              tmAlog, tmB, tmBlo, p));
  return SPMM_OK;
}

}  // namespace spmm
