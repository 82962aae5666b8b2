// The tuner's configuration space, the exhaustive sweeps over it, and the
// device-array wrapper of the structure features.
//
// The table has 56 entries:
//   * five mma.sync tiles (column tile x ring depth);
//   * 32 variants of the 128-column tcgen05 pipeline (column tile, ring depth,
//     TMEM accumulators, static or work-queue schedule, split-K of 1, 2, 4
//     and, for the default 256-column tile, 8);
//   * eight with a four-group ring and one accumulator (256 and 512 columns,
//     static or queue, split-K 1 or 2), which only e4m3 instantiates (four
//     blocks per group share one scale tile);
//   * four of the 64-row pipeline (column tile x schedule);
//   * seven per-matrix plans (schedule 2) on the tcgen05 shapes without
//     split-K: run through spmm_bcsr_plan_create / _run_ex with the
//     inputs-ready chain, which is how a caller with a fixed matrix runs.
// Which entries have a kernel depends on the block height and the type;
// spmm_config_supported answers that without launching.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "internal.h"

namespace spmm {
namespace {

std::vector<spmm_config> make_table() {
  std::vector<spmm_config> t;
  auto add = [&](int kernel, int nt, int stages, int acc, int sched, int split) {
    spmm_config c;
    std::memset(&c, 0, sizeof(c));
    c.kernel = kernel;
    c.n_tile = nt;
    c.stages = stages;
    c.acc_buffers = acc;
    c.schedule = sched;
    c.split_k = split;
    t.push_back(c);
  };
  add(1, 64, 4, 0, 0, 0);
  add(1, 128, 4, 0, 0, 0);
  add(1, 128, 8, 0, 0, 0);
  add(1, 256, 4, 0, 0, 0);
  add(1, 256, 8, 0, 0, 0);
  struct Tc {
    int nt, stages, acc, max_split;
  };
  const Tc tcs[] = {{128, 0, 2, 4}, {256, 0, 2, 8}, {256, 2, 2, 4}, {512, 0, 1, 4}, {512, 0, 2, 4}};
  for (const Tc& x : tcs)
    for (int sched = 0; sched < 2; ++sched)
      for (int split = 1; split <= x.max_split; split *= 2) add(2, x.nt, x.stages, x.acc, sched, split);
  // the 64-row pipeline with M = 64 UMMAs (64-row blocks only, no split-K)
  for (int nt : {256, 512})
    for (int sched = 0; sched < 2; ++sched) add(3, nt, 0, 0, sched, 1);
  // four-group rings with one accumulator (the e4m3 kernels)
  for (int nt : {256, 512})
    for (int sched = 0; sched < 2; ++sched)
      for (int split = 1; split <= 2; split *= 2) add(2, nt, 4, 1, sched, split);
  // per-matrix plans
  const Tc plans[] = {{128, 0, 2, 1}, {256, 0, 2, 1}, {256, 2, 2, 1}, {512, 0, 1, 1}, {512, 0, 2, 1},
                      {256, 4, 1, 1}, {512, 4, 1, 1}};
  for (const Tc& x : plans) add(2, x.nt, x.stages, x.acc, 2, 1);
  return t;
}

const std::vector<spmm_config>& table() {
  static const std::vector<spmm_config> t = make_table();
  return t;
}

}  // namespace
}  // namespace spmm

using namespace spmm;

extern "C" {

int spmm_tune_config_count(void) { return (int)table().size(); }

spmm_status spmm_tune_config(int i, spmm_config* out) {
  if (!out || i < 0 || i >= (int)table().size()) return fail(SPMM_ERR_INVALID_ARG, "config index out of range");
  *out = table()[i];
  return SPMM_OK;
}

spmm_status spmm_config_supported(int bR, spmm_dtype dtype, int N, const spmm_config* cfg) {
  if (!cfg) return fail(SPMM_ERR_INVALID_ARG, "null config");
  bool ok = false;
  if (cfg->kernel == 1) ok = cfg->split_k <= 1 && cfg->schedule == 0 && mma_supported(bR, dtype, N, *cfg);
  else if (cfg->kernel == 2) ok = cfg->schedule >= 0 && cfg->schedule <= 2 && (cfg->schedule < 2 || cfg->split_k <= 1) &&
                                  tc_supported(bR, dtype, N, *cfg);
  else if (cfg->kernel == 3) ok = cfg->schedule >= 0 && cfg->schedule <= 1 && tc64_supported(bR, dtype, N, *cfg);
  return ok ? SPMM_OK : SPMM_ERR_UNSUPPORTED;
}

spmm_status spmm_default_config(int bR, spmm_dtype dtype, int N, spmm_config* out) {
  if (!out) return fail(SPMM_ERR_INVALID_ARG, "null config");
  spmm_config c;
  std::memset(&c, 0, sizeof(c));
  // spmm_bcsr_mm with no configuration: the tcgen05 pipeline for 64-row
  // blocks where it has a kernel (its first instantiation for the column tile:
  // two accumulators, static schedule), else the mma.sync pipeline (depth 4).
  // E4M3 stays on mma.sync, which takes any fp32 block scale (the tcgen05
  // e4m3 kernels need powers of two).
  if (bR == 64 && dtype != SPMM_E4M3 && tc_supported(bR, dtype, N, c)) {
    c.kernel = 2;
    c.n_tile = N <= 128 ? 128 : 256;
    c.acc_buffers = 2;
    c.split_k = 1;
  } else {
    c.kernel = 1;
    c.n_tile = mma_default_nt(bR, dtype, N);
    c.stages = 4;
  }
  *out = c;
  return spmm_config_supported(bR, dtype, N, &c) == SPMM_OK ? SPMM_OK
                                                            : fail(SPMM_ERR_UNSUPPORTED, "no default kernel");
}

spmm_status spmm_tune_sweep(const spmm_bcsr_desc* A, const spmm_dense_desc* B, int N, float* C, int ldc,
                            int warmup, int reps, void* flush, size_t flush_bytes, float* ms_out,
                            void* stream) {
  if (!A || !B || !ms_out || reps < 1 || warmup < 0) return fail(SPMM_ERR_INVALID_ARG, "bad sweep arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  SPMM_CUDA_TRY(cudaEventCreate(&e0));
  SPMM_CUDA_TRY(cudaEventCreate(&e1));
  std::vector<float> ts(reps);
  spmm_status result = SPMM_OK;
  for (size_t i = 0; i < table().size() && result == SPMM_OK; ++i) {
    const spmm_config& c = table()[i];
    if (spmm_config_supported(A->bR, A->dtype, N, &c) != SPMM_OK) {
      ms_out[i] = INFINITY;
      continue;
    }
    // a plan entry times the plan's runs (one launch each, no early start:
    // every run follows an L2 flush)
    spmm_bcsr_plan* plan = nullptr;
    if (c.schedule == 2 && spmm_bcsr_plan_create(A, N, &c, stream, &plan) != SPMM_OK) {
      clear_error();
      ms_out[i] = INFINITY;
      continue;
    }
    auto run = [&]() {
      return plan ? spmm_bcsr_plan_run(plan, A, B, N, C, ldc, stream) : spmm_bcsr_mm(A, B, N, C, ldc, &c, stream);
    };
    for (int w = 0; w < warmup && result == SPMM_OK; ++w) result = run();
    for (int k = 0; k < reps && result == SPMM_OK; ++k) {
      if (flush && flush_bytes) {
        cudaError_t ce = cudaMemsetAsync(flush, k & 0xff, flush_bytes, s);
        if (ce != cudaSuccess) result = cuda_fail(ce, "flushing L2");
      }
      cudaEventRecord(e0, s);
      if (result == SPMM_OK) result = run();
      cudaEventRecord(e1, s);
      cudaError_t ce = cudaEventSynchronize(e1);
      if (ce != cudaSuccess && result == SPMM_OK) result = cuda_fail(ce, "timing a configuration");
      if (result == SPMM_OK) cudaEventElapsedTime(&ts[k], e0, e1);
    }
    if (plan) {
      cudaStreamSynchronize(s);
      spmm_bcsr_plan_destroy(plan);
    }
    if (result == SPMM_OK) {
      // the mean: event timestamps advance in steps of about 2 us on this
      // hardware, which a median would keep and a mean averages out
      double sum = 0;
      for (float x : ts) sum += x;
      ms_out[i] = (float)(sum / reps);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return result;
}

spmm_status spmm_tune_sweep_b2b(const spmm_problem* copies, int ncopies, int launches, int warmup, float* ms_out,
                                void* stream) {
  clear_error();
  if (!copies || ncopies < 1 || launches < 1 || warmup < 0 || !ms_out)
    return fail(SPMM_ERR_INVALID_ARG, "bad sweep arguments");
  const spmm_problem& P0 = copies[0];
  for (int k = 1; k < ncopies; ++k) {
    const spmm_problem& P = copies[k];
    if (P.A.M != P0.A.M || P.A.K != P0.A.K || P.A.bR != P0.A.bR || P.A.dtype != P0.A.dtype || P.N != P0.N)
      return fail(SPMM_ERR_INVALID_ARG, "the copies must be one problem (shape, block shape, type, N)");
  }
  // The sweep runs on a stream of its own (capture needs a stream other than
  // the legacy default one), ordered after the caller's work.
  cudaStream_t user = static_cast<cudaStream_t>(stream), s = nullptr;
  SPMM_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  spmm_status result = SPMM_OK;
  auto check = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && result == SPMM_OK) result = cuda_fail(e, what);
    return e == cudaSuccess;
  };
  check(cudaEventCreate(&e0), "cudaEventCreate");
  check(cudaEventCreate(&e1), "cudaEventCreate");
  if (result == SPMM_OK) {
    check(cudaEventRecord(e0, user), "cudaEventRecord");
    check(cudaStreamWaitEvent(s, e0, 0), "cudaStreamWaitEvent");
  }
  for (size_t i = 0; i < table().size() && result == SPMM_OK; ++i) {
    const spmm_config& c = table()[i];
    if (spmm_config_supported(P0.A.bR, P0.A.dtype, P0.N, &c) != SPMM_OK) {
      ms_out[i] = INFINITY;
      continue;
    }
    spmm_bcsr_plan* plan = nullptr;
    if (c.schedule == 2 && spmm_bcsr_plan_create(&P0.A, P0.N, &c, s, &plan) != SPMM_OK) {
      clear_error();
      ms_out[i] = INFINITY;
      continue;
    }
    // A plan's runs chain with the inputs-ready flag: inside the graph only
    // these products run, and none writes an A or a B.
    auto run = [&](int k, unsigned flags) {
      const spmm_problem& P = copies[k % ncopies];
      return plan ? spmm_bcsr_plan_run_ex(plan, &P.A, &P.B, P.N, P.C, P.ldc, flags, s)
                  : spmm_bcsr_mm(&P.A, &P.B, P.N, P.C, P.ldc, &c, s);
    };
    // eager warm-up: sets up what the library allocates lazily before capture
    for (int w = 0; w < std::max(warmup, 1) && result == SPMM_OK; ++w) result = run(w, 0u);
    if (result == SPMM_OK) check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool captured = false;
    if (result == SPMM_OK && cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
      spmm_status st = SPMM_OK;
      for (int k = 0; k < launches && st == SPMM_OK; ++k) st = run(k, plan ? SPMM_RUN_INPUTS_READY : 0u);
      const cudaError_t ec = cudaStreamEndCapture(s, &graph);
      captured = st == SPMM_OK && ec == cudaSuccess && graph &&
                 cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
      if (!captured) clear_error();
    }
    cudaGetLastError();   // clears the (non-sticky) error a failed capture leaves
    if (result == SPMM_OK && captured) check(cudaGraphLaunch(exec, s), "cudaGraphLaunch");   // upload
    if (result == SPMM_OK) check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (result == SPMM_OK) {
      check(cudaEventRecord(e0, s), "cudaEventRecord");
      if (captured) {
        check(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
      } else {   // no graph: the same launches issued one by one
        for (int k = 0; k < launches && result == SPMM_OK; ++k) result = run(k, plan ? SPMM_RUN_INPUTS_READY : 0u);
      }
      check(cudaEventRecord(e1, s), "cudaEventRecord");
      if (check(cudaEventSynchronize(e1), "timing a configuration")) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_out[i] = ms / launches;
      }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (plan) {
      cudaStreamSynchronize(s);
      spmm_bcsr_plan_destroy(plan);
    }
  }
  cudaStreamSynchronize(s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  return result;
}

spmm_status spmm_structure_features(const spmm_bcsr_desc* A, int N, float* out, void* stream) {
  if (!A || !out || !A->row_ptr || A->bR <= 0 || A->M <= 0 || A->M % A->bR)
    return fail(SPMM_ERR_INVALID_ARG, "bad features arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int MB = A->M / A->bR;
  std::vector<int> rp(MB + 1);
  SPMM_CUDA_TRY(cudaMemcpyAsync(rp.data(), A->row_ptr, sizeof(int) * (MB + 1), cudaMemcpyDeviceToHost, s));
  SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  if (rp[0] != 0 || rp[MB] < 0) return fail(SPMM_ERR_BAD_STRUCTURE, "row_ptr[0] != 0");
  const long long nnzb = rp[MB];
  std::vector<int> ci((size_t)std::max<long long>(nnzb, 1));
  if (nnzb > 0) {
    if (!A->col_idx) return fail(SPMM_ERR_INVALID_ARG, "null col_idx");
    SPMM_CUDA_TRY(cudaMemcpyAsync(ci.data(), A->col_idx, sizeof(int) * nnzb, cudaMemcpyDeviceToHost, s));
    SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (spmm_structure_features_host(rp.data(), ci.data(), A->M, A->K, A->bR, N, A->dtype, out) != 0)
    return fail(SPMM_ERR_BAD_STRUCTURE, "row_ptr / col_idx out of range");
  return SPMM_OK;
}

}  // extern "C"
