// A per-matrix plan for the tcgen05 pipeline: an item list ordered heaviest
// first, with block rows far longer than the rest split into parts, taken by
// the CTAs from the plan's own work queue.
//
// A launch of k_bcsr_tc is bound by its longest CTA: one item is a block row
// (and column tile), and a CTA streams its blocks at a fixed rate, so a row
// many times longer than the average sets the time while other CTAs idle. The
// plan reads row_ptr once. A row longer than 3x the average load per CTA slot
// is cut into parts of about that load, run by different CTAs: part 0 zeroes
// the row's C tile while its MMAs run, and every part adds its tile into C
// with red.add once that is done. Rows not split store C directly, as without
// a plan; on rows of similar lengths (no row that long) the plan only orders
// the items.
//
// Each CTA starts on item blockIdx.x and takes every later item from the
// queue shortly before it has copied the current one, so CTAs that run faster
// (lighter items, or an SM they no longer share) take more of the lighter
// items at the end of the list. Claims follow list order, and so does each
// CTA's own sequence of items.
//
// Stacking (16- and 32-row blocks): the tcgen05 UMMA costs the same for a
// block height of 16, 32 or 64, and every block loads its own B panel. When
// the 4 (or 2) block rows that make up 64 rows of C share most of their block
// columns (band and block-diagonal structures), the plan stacks them: the
// union of their columns becomes one 64-row BCSR row whose blocks hold the
// member rows' blocks and zeros, so one UMMA and one B panel serve 4 (or 2)
// blocks. A run is one launch of the 64-row pipeline whose B-panel issuers
// also copy each stacked block's member blocks from A's own values into the
// stage (a member row with no block reads a box past the end of A: zeros), so
// every run takes the current values. The plan stacks only when the union
// saves at least 40 % of the panels and N is above 256. Measured on 8192^2
// band and block-diagonal products at 20 %: at N = 512 stacking ran 1.0-1.24x
// faster as one cold launch and 1.07-1.46x back to back; at N = 256 it ran
// 0.87-1.0x cold, 16-row products 1.23-1.25x back to back and 32-row ones
// 0.93-0.95x. (A version that built the stacked blocks with a copy kernel
// before each run needed N above 512.)
//
// The plan holds only what row_ptr (and, for a stacked plan, col_idx)
// determines: any A with the same M, K, block shape, dtype and structure
// (values may change; column indices too for a plan that does not stack) runs
// on it.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>
#include "internal.h"

struct spmm_bcsr_plan {
  int M = 0, K = 0, bR = 0, N = 0;
  spmm_dtype dtype = SPMM_F16;
  spmm_config cfg{};
  int n_items = 0, n_pairs = 0;
  int4* items = nullptr;       // {block row, column tile, first block, end block}
  int* pair = nullptr;         // -1, or 128 * group + part
  int* parts = nullptr;        // parts per group (split row and tile)
  unsigned* counters = nullptr;   // per group: {C tile zeroed, parts finished}; then the queue
  unsigned* queue = nullptr;      // {next ticket, CTAs done}, inside `counters`
  // stacking: `stack` block rows per 64-row row (1: none)
  int stack = 1;
  long long stacked_blocks = 0;
  int* s_row_ptr = nullptr;       // M/64 + 1
  int* s_col_idx = nullptr;       // stacked_blocks
  int* s_map = nullptr;           // stacked_blocks x stack: source block of each member row, or -1
};

namespace spmm {
namespace {

constexpr int kMinPartBlocks = 8;   // shorter parts are not worth a hand-off
constexpr int kSplitFactor = 3;     // split rows longer than 3x the average load per CTA slot
constexpr int kMaxParts = 64;
constexpr int kStackKeepPct = 60;   // stack when the union has at most 60 % of the blocks
constexpr int kStackMinN = 256;     // and N is larger

// The stacked structure of 16- or 32-row blocks: for each group of `st` block
// rows (64 rows of C), the sorted union of their block columns, and per union
// column the block of each member row (or -1). False when a row repeats a
// column (the stacked block could not hold both).
bool build_stack(const int* rp, const int* ci, int MB, int st, std::vector<int>* srp, std::vector<int>* sci,
                 std::vector<int>* smap) {
  const int MS = MB / st;
  srp->assign(1, 0);
  sci->clear();
  smap->clear();
  std::vector<std::pair<int, int>> ent;   // (column, entry) of the group's blocks
  std::vector<int> member, block;         // per entry: member row, source block
  for (int g = 0; g < MS; ++g) {
    ent.clear();
    member.clear();
    block.clear();
    for (int t = 0; t < st; ++t) {
      const int r = g * st + t;
      for (int b = rp[r]; b < rp[r + 1]; ++b) {
        ent.push_back({ci[b], (int)member.size()});
        member.push_back(t);
        block.push_back(b);
      }
    }
    std::sort(ent.begin(), ent.end());
    for (size_t i = 0; i < ent.size();) {
      const int c = ent[i].first;
      const size_t base = smap->size();
      smap->resize(base + st, -1);
      for (; i < ent.size() && ent[i].first == c; ++i) {
        const int k = ent[i].second;
        if ((*smap)[base + member[k]] >= 0) return false;   // a row repeats a column
        (*smap)[base + member[k]] = block[k];
      }
      sci->push_back(c);
    }
    srp->push_back((int)sci->size());
  }
  return true;
}

}  // namespace

bool stack_structure_host(const int* rp, const int* ci, int MB, int st, std::vector<int>* srp, std::vector<int>* sci,
                          std::vector<int>* smap) {
  return build_stack(rp, ci, MB, st, srp, sci, smap);
}

namespace {

struct Item {
  int4 d;    // {block row, column tile, first block, end block}
  int pair;  // -1, or 128 * group + part
  int key;   // heaviness: its blocks, or for a part the longest part of its row
};

// The item list for row_ptr (MB + 1 entries), ntiles column tiles and
// `capacity` CTA slots: rows far above the average load per slot cut into
// parts, every item keyed by its heaviness, sorted heaviest first. Host code
// only; the device plan and spmm_bcsr_plan_items both use it.
void build_items(const int* rp, int MB, int ntiles, long long capacity, std::vector<Item>* out,
                 std::vector<int>* group_parts) {
  std::vector<Item>& items = *out;
  items.clear();
  group_parts->clear();
  long long total = 0;
  for (int r = 0; r < MB; ++r) total += (long long)(rp[r + 1] - rp[r]) * ntiles;
  const long long avg = std::max<long long>(kMinPartBlocks, (total + capacity - 1) / capacity);
  items.reserve((size_t)MB * ntiles + 64);
  for (int r = 0; r < MB; ++r) {
    const int len = rp[r + 1] - rp[r];
    const int k = len > kSplitFactor * avg ? (int)std::min<long long>(kMaxParts, (len + avg - 1) / avg) : 1;
    for (int t = 0; t < ntiles; ++t) {
      if (k == 1) {
        items.push_back({make_int4(r, t, rp[r], rp[r + 1]), -1, len});
        continue;
      }
      const int g = (int)group_parts->size();
      group_parts->push_back(k);
      for (int q = 0; q < k; ++q)
        items.push_back({make_int4(r, t, rp[r] + (int)((long long)len * q / k), rp[r] + (int)((long long)len * (q + 1) / k)),
                         128 * g + q, (len + k - 1) / k});
    }
  }
  // Heaviest first: with more items than CTAs, each CTA's next item is lighter.
  // The parts of a row share one key, so the stable sort keeps part 0 ahead of
  // its siblings: a CTA takes its items in list order, so every part waits only
  // for a part 0 earlier in the list, and those waits cannot form a cycle.
  std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& b) { return a.key > b.key; });
}

void plan_free(spmm_bcsr_plan* p) {
  if (!p) return;
  cudaFree(p->items);
  cudaFree(p->pair);
  cudaFree(p->parts);
  cudaFree(p->counters);
  cudaFree(p->s_row_ptr);
  cudaFree(p->s_col_idx);
  cudaFree(p->s_map);
  delete p;
}

}  // namespace
}  // namespace spmm

using namespace spmm;

extern "C" spmm_status spmm_bcsr_plan_create(const spmm_bcsr_desc* A, int N, const spmm_config* cfg, void* stream,
                                             spmm_bcsr_plan** out) {
  if (!out) return fail(SPMM_ERR_INVALID_ARG, "null output");
  *out = nullptr;
  if (!A) return fail(SPMM_ERR_INVALID_ARG, "null descriptor");
  if (A->M <= 0 || A->K <= 0 || N <= 0) return fail(SPMM_ERR_INVALID_ARG, "a plan needs a non-empty product");
  if (A->bC != 16 || (A->bR != 16 && A->bR != 32 && A->bR != 64))
    return fail(SPMM_ERR_UNSUPPORTED, "block shape must be 16, 32 or 64 x 16");
  if (A->M % A->bR || A->K % 16) return fail(SPMM_ERR_INVALID_ARG, "M / K not multiples of the block shape");
  if (N % 8) return fail(SPMM_ERR_UNSUPPORTED, "N must be a multiple of 8");
  if (!A->row_ptr) return fail(SPMM_ERR_INVALID_ARG, "null row_ptr");
  spmm_config c;
  std::memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if (c.kernel != 0 && c.kernel != 2) return fail(SPMM_ERR_UNSUPPORTED, "a plan runs on kernel 2");
  if (c.split_k > 1 || c.schedule < 0 || c.schedule > 2)
    return fail(SPMM_ERR_UNSUPPORTED, "a plan replaces split-K and brings its own work queue");
  c.kernel = 2;
  c.schedule = 1;   // the plan's queue
  const int MB = A->M / A->bR;
  std::vector<int> rp(MB + 1);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SPMM_CUDA_TRY(cudaMemcpyAsync(rp.data(), A->row_ptr, sizeof(int) * (MB + 1), cudaMemcpyDeviceToHost, s));
  SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  for (int r = 0; r < MB; ++r)
    if (rp[r + 1] < rp[r]) return fail(SPMM_ERR_INVALID_ARG, "row_ptr must not decrease");
  // stacking of 16- and 32-row blocks into the 64-row pipeline
  int st = 1, nt = 0, per_sm = 0;
  std::vector<int> srp, sci, smap;
  const long long nnzb = rp[MB];
  if ((A->bR == 16 || A->bR == 32) && A->M % 64 == 0 && N > kStackMinN &&
      (A->dtype == SPMM_F16 || A->dtype == SPMM_BF16) && nnzb > 0 && A->col_idx && A->vals &&
      tc_geometry(64, A->dtype, N, c, &nt, &per_sm)) {
    std::vector<int> ci((size_t)nnzb);
    SPMM_CUDA_TRY(cudaMemcpyAsync(ci.data(), A->col_idx, sizeof(int) * nnzb, cudaMemcpyDeviceToHost, s));
    SPMM_CUDA_TRY(cudaStreamSynchronize(s));
    const int cand = 64 / A->bR;
    if (build_stack(rp.data(), ci.data(), MB, cand, &srp, &sci, &smap) &&
        (long long)sci.size() * 100 <= nnzb * kStackKeepPct)
      st = cand;
  }
  if (st == 1 && !tc_geometry(A->bR, A->dtype, N, c, &nt, &per_sm))
    return fail(SPMM_ERR_UNSUPPORTED, "no tcgen05 kernel for this block height, dtype and configuration");
  c.n_tile = nt;
  const int rows = st > 1 ? A->M / 64 : MB;
  const int ntiles = (N + nt - 1) / nt;
  const long long capacity = (long long)sm_count() * per_sm;
  std::vector<Item> items;
  std::vector<int> group_parts;
  build_items(st > 1 ? srp.data() : rp.data(), rows, ntiles, capacity, &items, &group_parts);
  const int pairs = (int)group_parts.size();
  if (items.size() >= (1u << 30)) return fail(SPMM_ERR_UNSUPPORTED, "too many work items");
  std::vector<int4> hd(items.size());
  std::vector<int> hp(items.size());
  for (size_t i = 0; i < items.size(); ++i) {
    hd[i] = items[i].d;
    hp[i] = items[i].pair;
  }
  spmm_bcsr_plan* p = new spmm_bcsr_plan;
  p->M = A->M;
  p->K = A->K;
  p->bR = A->bR;
  p->N = N;
  p->dtype = A->dtype;
  p->cfg = c;
  p->n_items = (int)items.size();
  p->n_pairs = pairs;
  if (cudaMalloc(&p->items, sizeof(int4) * hd.size()) != cudaSuccess ||
      cudaMalloc(&p->pair, sizeof(int) * hp.size()) != cudaSuccess ||
      cudaMalloc(&p->parts, sizeof(int) * std::max(pairs, 1)) != cudaSuccess ||
      cudaMalloc(&p->counters, sizeof(unsigned) * (2 * std::max(pairs, 1) + 2)) != cudaSuccess) {
    plan_free(p);
    return fail(SPMM_ERR_CUDA, "plan allocation failed");
  }
  if (cudaMemcpy(p->items, hd.data(), sizeof(int4) * hd.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->pair, hp.data(), sizeof(int) * hp.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      (pairs > 0 && cudaMemcpy(p->parts, group_parts.data(), sizeof(int) * pairs, cudaMemcpyHostToDevice) != cudaSuccess) ||
      cudaMemset(p->counters, 0, sizeof(unsigned) * (2 * std::max(pairs, 1) + 2)) != cudaSuccess) {
    plan_free(p);
    return fail(SPMM_ERR_CUDA, "plan upload failed");
  }
  p->queue = p->counters + 2 * std::max(pairs, 1);
  if (st > 1) {
    // the stacked structure: row pointers, column indices and member map
    p->stack = st;
    p->stacked_blocks = (long long)sci.size();
    if (cudaMalloc(&p->s_row_ptr, sizeof(int) * srp.size()) != cudaSuccess ||
        cudaMalloc(&p->s_col_idx, sizeof(int) * sci.size()) != cudaSuccess ||
        cudaMalloc(&p->s_map, sizeof(int) * smap.size()) != cudaSuccess) {
      plan_free(p);
      return fail(SPMM_ERR_CUDA, "stacked plan allocation failed");
    }
    if (cudaMemcpy(p->s_row_ptr, srp.data(), sizeof(int) * srp.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(p->s_col_idx, sci.data(), sizeof(int) * sci.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(p->s_map, smap.data(), sizeof(int) * smap.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      plan_free(p);
      return fail(SPMM_ERR_CUDA, "stacked plan upload failed");
    }
  }
  *out = p;
  return SPMM_OK;
}

extern "C" spmm_status spmm_bcsr_plan_stacking(const spmm_bcsr_plan* p, int* rows_per_stack, long long* blocks) {
  if (!p) return fail(SPMM_ERR_INVALID_ARG, "null plan");
  if (rows_per_stack) *rows_per_stack = p->stack;
  if (blocks) *blocks = p->stacked_blocks;
  return SPMM_OK;
}

extern "C" spmm_status spmm_bcsr_plan_info(const spmm_bcsr_plan* p, int* items, int* split_rows, spmm_config* cfg) {
  if (!p) return fail(SPMM_ERR_INVALID_ARG, "null plan");
  if (items) *items = p->n_items;
  if (split_rows) *split_rows = p->n_pairs;
  if (cfg) *cfg = p->cfg;
  return SPMM_OK;
}

extern "C" spmm_status spmm_bcsr_plan_run(const spmm_bcsr_plan* p, const spmm_bcsr_desc* A, const spmm_dense_desc* B,
                                          int N, float* C, int ldc, void* stream) {
  return spmm_bcsr_plan_run_ex(p, A, B, N, C, ldc, 0u, stream);
}

extern "C" spmm_status spmm_bcsr_plan_run_ex(const spmm_bcsr_plan* p, const spmm_bcsr_desc* A,
                                             const spmm_dense_desc* B, int N, float* C, int ldc, unsigned flags,
                                             void* stream) {
  if (!p || !A || !B) return fail(SPMM_ERR_INVALID_ARG, "null plan or descriptor");
  if (flags & ~SPMM_RUN_INPUTS_READY) return fail(SPMM_ERR_INVALID_ARG, "unknown run flags");
  if (A->M != p->M || A->K != p->K || A->bR != p->bR || A->dtype != p->dtype || N != p->N)
    return fail(SPMM_ERR_INVALID_ARG, "A and N must match the plan");
  if (!A->row_ptr || !C || !B->data) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  if (B->ldb < N || B->ldb % 8) return fail(SPMM_ERR_MISALIGNED, "ldb must be >= N and a multiple of 8");
  if (ldc < N || ldc % 4) return fail(SPMM_ERR_MISALIGNED, "ldc must be >= N and a multiple of 4");
  auto al16 = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  if ((A->vals && !al16(A->vals)) || !al16(B->data) || !al16(C))
    return fail(SPMM_ERR_MISALIGNED, "A values, B and C must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  spmm_bcsr_desc a64;
  const spmm_bcsr_desc* Arun = A;
  if (p->stack > 1) {
    // the 64-row pipeline over the stacked structure; its stacked blocks are
    // assembled in the stage from this A's member blocks
    if (!A->vals) return fail(SPMM_ERR_INVALID_ARG, "null values");
    a64 = *A;
    a64.bR = 64;
    a64.row_ptr = p->s_row_ptr;
    a64.col_idx = p->s_col_idx;
    a64.vals_lo = nullptr;
    a64.scales = nullptr;
    Arun = &a64;
  }
  LaunchRequest r;
  r.A = Arun;
  r.B = B;
  r.N = N;
  r.C = C;
  r.ldc = ldc;
  r.cfg = p->cfg;
  r.stream = s;
  r.items = p->items;
  r.pair = p->n_pairs > 0 ? p->pair : nullptr;
  r.parts = p->parts;
  r.counters = p->counters;
  r.plan_items = p->n_items;
  r.queue = p->queue;
  r.inputs_ready = (flags & SPMM_RUN_INPUTS_READY) != 0;
  if (p->stack > 1) {
    r.stack_map = p->s_map;
    r.stack = p->stack;
    r.member_bR = p->bR;
  }
  return launch_tc(r);
}

extern "C" spmm_status spmm_bcsr_plan_destroy(spmm_bcsr_plan* p) {
  plan_free(p);
  return SPMM_OK;
}

extern "C" spmm_status spmm_bcsr_plan_items(const int* row_ptr, int MB, int ntiles, long long slots, int* n_items,
                                            int* n_groups, int* items, int* pair, int* parts) {
  if (!row_ptr || MB < 0 || ntiles < 1 || slots < 1 || !n_items || !n_groups)
    return fail(SPMM_ERR_INVALID_ARG, "bad plan-items arguments");
  for (int r = 0; r < MB; ++r)
    if (row_ptr[r + 1] < row_ptr[r]) return fail(SPMM_ERR_INVALID_ARG, "row_ptr must not decrease");
  std::vector<Item> list;
  std::vector<int> group_parts;
  build_items(row_ptr, MB, ntiles, slots, &list, &group_parts);
  if (list.size() >= (1u << 30)) return fail(SPMM_ERR_UNSUPPORTED, "too many work items");
  *n_items = (int)list.size();
  *n_groups = (int)group_parts.size();
  for (size_t i = 0; i < list.size(); ++i) {
    if (items) {
      items[4 * i] = list[i].d.x;
      items[4 * i + 1] = list[i].d.y;
      items[4 * i + 2] = list[i].d.z;
      items[4 * i + 3] = list[i].d.w;
    }
    if (pair) pair[i] = list[i].pair;
  }
  if (parts)
    for (size_t g = 0; g < group_parts.size(); ++g) parts[g] = group_parts[g];
  return SPMM_OK;
}

extern "C" spmm_status spmm_bcsr_stack_structure(const int* row_ptr, const int* col_idx, int MB, int rows_per_stack,
                                                 long long* stacked_blocks, int* s_row_ptr, int* s_col_idx,
                                                 int* s_map) {
  if (!row_ptr || MB < 0 || rows_per_stack < 1 || MB % rows_per_stack || !stacked_blocks)
    return fail(SPMM_ERR_INVALID_ARG, "bad stacking arguments");
  for (int r = 0; r < MB; ++r)
    if (row_ptr[r + 1] < row_ptr[r]) return fail(SPMM_ERR_INVALID_ARG, "row_ptr must not decrease");
  if (row_ptr[MB] > 0 && !col_idx) return fail(SPMM_ERR_INVALID_ARG, "null col_idx");
  std::vector<int> srp, sci, smap;
  if (!build_stack(row_ptr, col_idx, MB, rows_per_stack, &srp, &sci, &smap))
    return fail(SPMM_ERR_INVALID_ARG, "a block row repeats a column");
  *stacked_blocks = (long long)sci.size();
  if (s_row_ptr) std::copy(srp.begin(), srp.end(), s_row_ptr);
  if (s_col_idx) std::copy(sci.begin(), sci.end(), s_col_idx);
  if (s_map) std::copy(smap.begin(), smap.end(), s_map);
  return SPMM_OK;
}
