// Host-side internals shared by the translation units of libbcsr_spmm.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "../../include/bcsr_spmm.h"

namespace spmm {

// Thread-local last-error text; returns the status for chaining.
spmm_status fail(spmm_status st, const std::string& msg);
spmm_status cuda_fail(cudaError_t e, const char* what);
void clear_error();                              // empties the calling thread's last-error text
#define SPMM_CUDA_TRY(expr)                                   \
  do {                                                        \
    cudaError_t _e = (expr);                                  \
    if (_e != cudaSuccess) return ::spmm::cuda_fail(_e, #expr); \
  } while (0)

int sm_count();                                  // SMs of the current device
int smem_per_sm();                               // shared memory per SM of the current device (bytes)
// Sets a kernel's dynamic shared-memory limit once per device (cached).
cudaError_t ensure_smem_attr(const void* fn, int bytes);
// Occupancy query, cached per (kernel, device, block, smem).
int max_blocks_per_sm(const void* fn, int threads, size_t smem);

// Programmatic dependent launch (on unless SPMM_NO_PDL is set): the library's
// pipeline kernels wait (griddepcontrol.wait) before touching global memory,
// so they may start while the previous kernel in the stream finishes.
bool pdl_enabled();
template <typename... KArgs, typename... Args>
cudaError_t launch_kernel(void (*fn)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                          Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, static_cast<Args&&>(args)...);
}
unsigned* device_error_word();                   // per-device error word (lazy)
// A zeroed pair {next item, CTAs done} for one persistent launch's work queue.
// Slots rotate over a per-device pool; each launch's last CTA zeroes its slot
// again, so a slot is reusable as soon as the launch that used it has ended.
unsigned* work_queue_slot();

// cuTensorMapEncodeTiled through the runtime's driver entry point.
spmm_status encode_tile_map_2d(CUtensorMap* map, CUtensorMapDataType dt, const void* base,
                               uint64_t inner, uint64_t outer, uint64_t row_stride_bytes,
                               uint32_t box_inner, uint32_t box_outer, CUtensorMapSwizzle swz);

// B (K x N, row-major, 16-bit or 8-bit elements) as a 3-D tensor {W columns,
// K rows, N/W column blocks}, W = 128 bytes of columns (64 16-bit, 128 8-bit),
// with 128-byte swizzle and box {W, 16, boxes}: one TMA copy lands a 16-row
// panel of W*boxes columns as consecutive 2 KB atoms (the same shared-memory
// image as `boxes` separate W-column 2-D copies). Needs N % W == 0 so that no
// box column lies past the end of a row.
spmm_status encode_panel_map_3d(CUtensorMap* map, const void* base, uint64_t N, uint64_t K,
                                uint64_t row_stride_bytes, uint32_t boxes, int elem_bytes = 2);

struct LaunchRequest {
  const spmm_bcsr_desc* A;
  const spmm_dense_desc* B;
  int N;
  float* C;
  long long ldc;
  spmm_config cfg;
  cudaStream_t stream;
  // Caller-provided scratch (both NULL for every entry point except the
  // allocation-free one): the device error word and the work-queue pair.
  unsigned* err_word = nullptr;
  unsigned* queue = nullptr;
  // hybrid product: the CSR part added by the tcgen05 pipeline's epilogue
  const spmm_csr_desc* csr = nullptr;
  // planned hybrid product: A holds gather blocks (col_idx = -(g + 1)) whose
  // 16 B rows are gather_rows[16g .. 16g + 15]; total_blocks counts A's
  // stored and gather blocks
  const int* gather_rows = nullptr;
  long long total_blocks = 0;
  // planned product (kernel 2): the item list, split-row pairs and their
  // counters (see spmm_bcsr_plan_create)
  const int4* items = nullptr;
  const int* pair = nullptr;
  const int* parts = nullptr;
  unsigned* counters = nullptr;
  int plan_items = 0;
  // no kernel launched on the stream since its last host synchronisation
  // writes A or B: the pipeline's copies and MMAs may start before the
  // previous kernel has finished (plans only)
  bool inputs_ready = false;
  // stacked plan: A describes the 64-row stacked structure over the values of
  // the original member_bR-row blocks; each stacked block is `stack` members,
  // stack_map[block * stack + t] = member t's source block, or -1 (zeros)
  const int* stack_map = nullptr;
  int stack = 1;
  int member_bR = 0;
};
// The tcgen05 pipeline's column tile and CTAs per SM for a product (false when
// it has no kernel for it): what a plan builds its item list for.
bool tc_geometry(int bR, spmm_dtype dtype, int N, const spmm_config& cfg, int* nt, int* ctas_per_sm);
// mma.sync family (spmm_mma.cu)
spmm_status launch_mma(const LaunchRequest& r);
// tcgen05 family (spmm_tc.cu); returns SPMM_ERR_UNSUPPORTED when it has no kernel for r
spmm_status launch_tc(const LaunchRequest& r);
// tcgen05, 64-row blocks, M = 64 UMMAs (spmm_tc64.cu)
spmm_status launch_tc64(const LaunchRequest& r);

// Whether a pipeline has an instantiation for this block height, type, N and
// configuration (the same lookup its launcher makes).
bool mma_supported(int bR, spmm_dtype dtype, int N, const spmm_config& cfg);
bool tc_supported(int bR, spmm_dtype dtype, int N, const spmm_config& cfg);
bool tc64_supported(int bR, spmm_dtype dtype, int N, const spmm_config& cfg);
int mma_default_nt(int bR, spmm_dtype dtype, int N);   // the column tile spmm_bcsr_mm picks by default

unsigned long long wait_limit_ns();              // bounded-wait limit for device waits

// The stacked structure of 16- or 32-row blocks (bcsr_plan.cu): each group of
// `st` block rows becomes one 64-row row over the sorted union of their block
// columns; smap holds, per stacked block and member row, the source block or
// -1. False when a row repeats a column.
bool stack_structure_host(const int* rp, const int* ci, int MB, int st, std::vector<int>* srp, std::vector<int>* sci,
                          std::vector<int>* smap);

// row_ptr[0] = 0, row_ptr[i + 1] = counts[0] + ... + counts[i] (one CTA, asynchronous).
spmm_status scan_counts(const int* counts, int* row_ptr, int n, cudaStream_t s);

}  // namespace spmm
