// Instantiations and host dispatch of the mma.sync BCSR pipeline.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "internal.h"
#include "spmm_mma.cuh"

namespace spmm {
namespace {

using KernelFn = void (*)(const CUtensorMap, const CUtensorMap, const MmaParams);

struct Entry {
  int br, mode, nt, stages, wm, wn;
  KernelFn fn;
  size_t smem;
  int threads;
};

#define SPMM_MMA_ENTRY(BR, NT, WM, WN, ST, MODE)                                   \
  Entry{BR,                                                                        \
        MODE,                                                                      \
        NT,                                                                        \
        ST,                                                                        \
        WM,                                                                        \
        WN,                                                                        \
        &k_bcsr_mma<BR, NT, WM, WN, ST, MODE>,                                     \
        MmaCfg<BR, NT, WM, WN, ST, MODE>::kSmem,                                   \
        MmaCfg<BR, NT, WM, WN, ST, MODE>::kThreads}

// The configuration space the tuner sweeps (block height x column tile x depth).
#define SPMM_MMA_SHAPES(MODE)                                                      \
  SPMM_MMA_ENTRY(16, 64, 1, 4, 4, MODE), SPMM_MMA_ENTRY(16, 128, 1, 4, 4, MODE),    \
      SPMM_MMA_ENTRY(16, 128, 1, 4, 8, MODE), SPMM_MMA_ENTRY(16, 256, 1, 4, 4, MODE), \
      SPMM_MMA_ENTRY(16, 256, 1, 4, 8, MODE), SPMM_MMA_ENTRY(32, 64, 2, 2, 4, MODE),  \
      SPMM_MMA_ENTRY(32, 128, 2, 2, 4, MODE), SPMM_MMA_ENTRY(32, 128, 2, 2, 8, MODE), \
      SPMM_MMA_ENTRY(32, 256, 2, 2, 4, MODE), SPMM_MMA_ENTRY(64, 64, 4, 1, 4, MODE),  \
      SPMM_MMA_ENTRY(64, 128, 2, 2, 4, MODE), SPMM_MMA_ENTRY(64, 128, 2, 2, 8, MODE), \
      SPMM_MMA_ENTRY(64, 256, 2, 2, 4, MODE)

const Entry kEntries[] = {
    SPMM_MMA_SHAPES(MODE_F16),
    SPMM_MMA_SHAPES(MODE_BF16),
    SPMM_MMA_ENTRY(16, 128, 1, 4, 4, MODE_SPLIT),
    SPMM_MMA_ENTRY(32, 128, 2, 2, 4, MODE_SPLIT),
    SPMM_MMA_ENTRY(64, 128, 2, 2, 4, MODE_SPLIT),
    SPMM_MMA_ENTRY(64, 64, 4, 1, 4, MODE_SPLIT),
    SPMM_MMA_ENTRY(16, 128, 1, 4, 4, MODE_E4M3),
    SPMM_MMA_ENTRY(16, 256, 1, 4, 4, MODE_E4M3),
    SPMM_MMA_ENTRY(32, 128, 2, 2, 4, MODE_E4M3),
    SPMM_MMA_ENTRY(64, 128, 2, 2, 4, MODE_E4M3),
    SPMM_MMA_ENTRY(64, 256, 2, 2, 4, MODE_E4M3),
};

int mode_of(spmm_dtype d) {
  switch (d) {
    case SPMM_F16: return MODE_F16;
    case SPMM_BF16: return MODE_BF16;
    case SPMM_F16_SPLIT: return MODE_SPLIT;
    case SPMM_E4M3: return MODE_E4M3;
  }
  return -1;
}

// Default column tile when the caller does not pick one.
int default_nt(int br, int mode, int N) {
  if (mode == MODE_E4M3) return 128;
  if (mode == MODE_SPLIT) return br == 64 && N <= 64 ? 64 : 128;
  if (br == 16) return N >= 256 ? 256 : (N >= 128 ? 128 : 64);
  if (br == 32) return N >= 128 ? 128 : 64;
  return N >= 128 ? 128 : 64;
}

const Entry* find_entry(int br, int mode, int nt, int stages) {
  const Entry* best = nullptr;
  for (const Entry& e : kEntries) {
    if (e.br != br || e.mode != mode || e.nt != nt) continue;
    if (stages > 0 && e.stages != stages) continue;
    if (!best || (stages <= 0 && e.stages == 4)) best = &e;
  }
  return best;
}

}  // namespace

int mma_default_nt(int bR, spmm_dtype dtype, int N) {
  const int mode = mode_of(dtype);
  return mode < 0 ? 0 : default_nt(bR, mode, N);
}

bool mma_supported(int bR, spmm_dtype dtype, int N, const spmm_config& cfg) {
  const int mode = mode_of(dtype);
  if (mode < 0) return false;
  const int nt = cfg.n_tile > 0 ? cfg.n_tile : default_nt(bR, mode, N);
  return find_entry(bR, mode, nt, cfg.stages) != nullptr;
}

spmm_status launch_mma(const LaunchRequest& r) {
  const spmm_bcsr_desc& A = *r.A;
  const spmm_dense_desc& B = *r.B;
  const int mode = mode_of(A.dtype);
  if (mode < 0) return fail(SPMM_ERR_INVALID_ARG, "unknown dtype");
  const int nt = r.cfg.n_tile > 0 ? r.cfg.n_tile : default_nt(A.bR, mode, r.N);
  const Entry* e = find_entry(A.bR, mode, nt, r.cfg.stages);
  if (!e)
    return fail(SPMM_ERR_UNSUPPORTED, "no mma.sync kernel for bR=" + std::to_string(A.bR) +
                                          " n_tile=" + std::to_string(nt) +
                                          " stages=" + std::to_string(r.cfg.stages));
  const bool e4m3 = mode == MODE_E4M3;
  const int esz = e4m3 ? 1 : 2;
  CUtensorMap tmB, tmBlo;
  std::memset(&tmBlo, 0, sizeof(tmBlo));
  const CUtensorMapDataType dt = e4m3 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
  // 16-bit B panels: one 3-D copy per panel when N is a multiple of 64.
  int panel3d = (!e4m3 && r.N % 64 == 0) ? 1 : 0;
  spmm_status st = SPMM_OK;
  if (panel3d && encode_panel_map_3d(&tmB, B.data, (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * 2,
                                     (uint32_t)(nt / 64)) != SPMM_OK)
    panel3d = 0;
  if (!panel3d) {
    st = encode_tile_map_2d(&tmB, dt, B.data, (uint64_t)r.N, (uint64_t)A.K, (uint64_t)B.ldb * esz,
                            128 / esz, 16, CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  }
  if (mode == MODE_SPLIT) {
    st = panel3d ? encode_panel_map_3d(&tmBlo, B.data_lo, (uint64_t)r.N, (uint64_t)A.K,
                                       (uint64_t)B.ldb * 2, (uint32_t)(nt / 64))
                 : encode_tile_map_2d(&tmBlo, dt, B.data_lo, (uint64_t)r.N, (uint64_t)A.K,
                                      (uint64_t)B.ldb * esz, 128 / esz, 16, CU_TENSOR_MAP_SWIZZLE_128B);
    if (st != SPMM_OK) return st;
  } else {
    tmBlo = tmB;
  }

  MmaParams p;
  p.row_ptr = A.row_ptr;
  p.col_idx = A.col_idx;
  p.vals = static_cast<const uint8_t*>(A.vals);
  p.vals_lo = static_cast<const uint8_t*>(A.vals_lo);
  p.scales = A.scales;
  p.C = r.C;
  p.ldc = r.ldc;
  p.MB = A.M / A.bR;
  p.N = r.N;
  p.ntiles = (r.N + nt - 1) / nt;
  p.n_items = p.MB * p.ntiles;
  p.b_scale = B.scale;
  p.timeout_ns = wait_limit_ns();
  p.err = device_error_word();
  p.panel3d = panel3d;
  if (!p.err) return fail(SPMM_ERR_CUDA, "could not set up the device error word");
  if (p.n_items == 0) return SPMM_OK;

  SPMM_CUDA_TRY(ensure_smem_attr(reinterpret_cast<const void*>(e->fn), (int)e->smem));
  int per_sm = r.cfg.ctas_per_sm;
  if (per_sm <= 0) {
    per_sm = max_blocks_per_sm(reinterpret_cast<const void*>(e->fn), e->threads, e->smem);
    if (per_sm < 1) per_sm = 1;
  }
  long long grid = (long long)sm_count() * per_sm;
  if (grid > p.n_items) grid = p.n_items;
  if (std::getenv("SPMM_DEBUG"))
    std::fprintf(stderr, "[spmm] mma.sync bR=%d nt=%d stages=%d smem=%zu per_sm=%d grid=%lld items=%d\n",
                 A.bR, nt, e->stages, e->smem, per_sm, grid, p.n_items);
  SPMM_CUDA_TRY(launch_kernel(e->fn, dim3((unsigned)grid), dim3(e->threads), e->smem, r.stream, tmB, tmBlo, p));
  return SPMM_OK;
}

}  // namespace spmm
