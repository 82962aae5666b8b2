// Allocation-free variant of the BCSR product (spmm_bcsr_mm_noalloc).
//
// Some callers cannot call cudaMalloc: code running under a custom device
// allocator or a memory budget that forbids the CUDA allocator, plugins whose
// host application owns every device allocation, and code that must not
// allocate while a stream is being captured into a CUDA graph. The regular
// entry point allocates two small device buffers on first use (the device
// error word and the pool of work-queue counters); this variant takes its
// scratch from a fixed array compiled into the library instead.
//
// The array below is that scratch. It is a file-scope __device__ array, so
// every GPU that loads the library holds it until the process exits. Host code
// cannot use its name as a device address: the address comes from
// cudaGetSymbolAddress, once per device, with that device current, on the
// first call made on that device, and is kept for the rest of the process. A
// cudaDeviceReset unloads the module, and the array may come back at another
// address: do not use this variant on a device after resetting it.
#include <cstring>
#include <mutex>
#include "internal.h"

namespace spmm {
namespace {

// Word 0: device error word (set by a bounded wait that gave up).
// Words 1-2: the work queue's {next item, CTAs done} pair.
// The rest pads the array to its alignment.
constexpr int kScratchWords = 64;
static __device__ __align__(256) unsigned g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned* g_scratch_ptr[kMaxDevices] = {nullptr};

// The device address of this device's scratch (set-up on first use).
spmm_status scratch_for_current_device(unsigned** out) {
  int dev = 0;
  SPMM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(SPMM_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_ptr[dev] = static_cast<unsigned*>(ptr);
  }
  *out = g_scratch_ptr[dev];
  return SPMM_OK;
}

}  // namespace
}  // namespace spmm

using namespace spmm;

extern "C" {

spmm_status spmm_bcsr_mm_noalloc(const spmm_bcsr_desc* A, const spmm_dense_desc* B, int N, float* C,
                                 int ldc, const spmm_config* cfg, void* stream) {
  clear_error();
  if (!A || !B) return fail(SPMM_ERR_INVALID_ARG, "null descriptor");
  if (A->M < 0 || A->K < 0 || N < 0) return fail(SPMM_ERR_INVALID_ARG, "negative size");
  if (A->bC != 16) return fail(SPMM_ERR_UNSUPPORTED, "block width must be 16");
  if (A->bR != 16 && A->bR != 32 && A->bR != 64)
    return fail(SPMM_ERR_UNSUPPORTED, "block height must be 16, 32 or 64");
  if (A->M % A->bR) return fail(SPMM_ERR_INVALID_ARG, "M must be a multiple of the block height");
  if (A->K % 16) return fail(SPMM_ERR_INVALID_ARG, "K must be a multiple of 16");
  if (A->dtype != SPMM_F16 && A->dtype != SPMM_BF16 && A->dtype != SPMM_F16_SPLIT)
    return fail(SPMM_ERR_UNSUPPORTED, "the allocation-free variant runs fp16, bf16 and split fp16");
  if (A->M == 0 || N == 0) return SPMM_OK;
  if (!A->row_ptr || !C || !B->data) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  const bool split = A->dtype == SPMM_F16_SPLIT;
  if (split && (!A->vals_lo || !B->data_lo))
    return fail(SPMM_ERR_INVALID_ARG, "F16_SPLIT needs the low halves of A and B");
  if (N % 8) return fail(SPMM_ERR_UNSUPPORTED, "N must be a multiple of 8");
  if (B->ldb < N || B->ldb % 8) return fail(SPMM_ERR_MISALIGNED, "ldb must be >= N and a multiple of 8");
  if (ldc < N || ldc % 4) return fail(SPMM_ERR_MISALIGNED, "ldc must be >= N and a multiple of 4");
  auto al = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  if (!al(A->vals) || !al(B->data) || !al(C) || (split && (!al(A->vals_lo) || !al(B->data_lo))))
    return fail(SPMM_ERR_MISALIGNED, "A values, B and C must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (A->K == 0) {
    // no block columns: C = 0 over the window (a memset allocates nothing)
    SPMM_CUDA_TRY(cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, A->M, s));
    return SPMM_OK;
  }
  spmm_config run_cfg;
  std::memset(&run_cfg, 0, sizeof(run_cfg));
  if (cfg) run_cfg = *cfg;
  run_cfg.kernel = 2;
  run_cfg.schedule = 1;
  // The work items the launch will hold: block rows x column tiles of the
  // tile that runs x split-K slices. The queue counters are 32-bit and
  // overshoot the item count by up to the grid size, so a launch may hold
  // fewer than 2^30 items (the pipeline's own limit).
  int nt = 0, per_sm = 0;
  if (!tc_geometry(A->bR, A->dtype, N, run_cfg, &nt, &per_sm))
    return fail(SPMM_ERR_UNSUPPORTED, "no tcgen05 kernel for this block height, type and configuration");
  const long long items =
      (long long)(A->M / A->bR) * ((N + nt - 1) / nt) * (run_cfg.split_k > 1 ? run_cfg.split_k : 1);
  if (items >= (1ll << 30))
    return fail(SPMM_ERR_SCRATCH_TOO_SMALL,
                "problem has " + std::to_string(items) +
                    " work items; the allocation-free variant's 32-bit queue holds fewer than 2^30");

  unsigned* scratch = nullptr;
  spmm_status st = scratch_for_current_device(&scratch);
  if (st != SPMM_OK) return st;
  // Every call shares the array: the error word and the queue pair start at zero.
  SPMM_CUDA_TRY(cudaMemsetAsync(scratch, 0, 3 * sizeof(unsigned), s));

  LaunchRequest r;
  r.A = A;
  r.B = B;
  r.N = N;
  r.C = C;
  r.ldc = ldc;
  r.cfg = run_cfg;
  r.stream = s;
  r.err_word = scratch;
  r.queue = scratch + 1;
  return launch_tc(r);
}

spmm_status spmm_noalloc_error_check(void* stream) {
  clear_error();
  unsigned* scratch = nullptr;
  spmm_status st = scratch_for_current_device(&scratch);
  if (st != SPMM_OK) return st;
  SPMM_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  unsigned v = 0;
  SPMM_CUDA_TRY(cudaMemcpy(&v, scratch, sizeof(v), cudaMemcpyDeviceToHost));
  if (v) return fail(SPMM_ERR_TIMEOUT, "a device-side pipeline wait timed out (code " + std::to_string(v) + ")");
  return SPMM_OK;
}

}  // extern "C"
