// spmm_nvbench_benches: the reference's NVBench benches for the BCSR path
// (nvbench_main.cu:326-1414, registered at :1417-1449), written against the
// NVBench surface of nvbench_compat.cuh and this library's C++ drop-in classes
// and C-ABI launchers.
//
// Every bench keeps the reference bench's shape: axes M, K, N, SPARS (percent
// of zero blocks) and PAT (an index into the reference generator's pattern
// list); inputs from mg::generate_matrix (seeds 123 for A, 456 for B); A built
// as a BCSRMatrix and moved to the device with copyToDevice; C cleared on the
// launch stream and the launch timed with exec_tag::timer; after the
// measurement, the result compared with a host product at the reference's
// tolerance (1e-2 absolute), exiting non-zero on a mismatch. The launch is the
// library's launcher of the bench's name (sparseMatrixMulTensor*_launch), which
// chooses its own grid.
//
//   spmm_nvbench_benches [-l] [-b NAME] [-a 'M=[512]'] ... [--csv FILE]
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "bcsr_spmm.h"
#include "bcsr_spmm.hpp"
#include "nvbench_compat.cuh"

namespace {

// The reference harness's pattern list (nvbench_main.cu:56-64), indexed by PAT.
const std::vector<std::string> kPatterns = {"random",     "checkerboard",  "diagonal",     "blockdiagonal",
                                            "blockrandom", "pattern64by16", "pattern32by16"};

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    std::exit(2);
  }
}

// One problem's host matrices and device arrays, built the way the reference
// harness builds them (its prepare_buffers, nvbench_main.cu:139-175).
struct Problem {
  std::unique_ptr<Matrix> A, B;
  std::unique_ptr<BCSRMatrix> bcsr;
  int* hdr = nullptr;
  int* idx = nullptr;
  half* data = nullptr;
  half* dB = nullptr;
  float* dC = nullptr;
  int M = 0, K = 0, N = 0;
  ~Problem() {
    cudaFree(hdr);
    cudaFree(idx);
    cudaFree(data);
    cudaFree(dB);
    cudaFree(dC);
  }
};

void fill(Matrix& dst, const mg::Matrix<float>& src) {
  for (int i = 0; i < dst.rows; ++i)
    for (int j = 0; j < dst.cols; ++j) dst.data[(size_t)i * dst.cols + j] = __float2half(src[i][j]);
}

std::unique_ptr<Problem> make_problem(int M, int K, int N, double sparsity, const std::string& pattern, int bR) {
  auto p = std::make_unique<Problem>();
  p->M = M;
  p->K = K;
  p->N = N;
  p->A = std::make_unique<Matrix>(M, K);
  p->B = std::make_unique<Matrix>(K, N);
  fill(*p->A, mg::generate_matrix<float>(M, K, sparsity, pattern, bR, 123));
  fill(*p->B, mg::generate_matrix<float>(K, N, 0.0, "random", bR, 456));
  p->bcsr = std::make_unique<BCSRMatrix>(*p->A, bR, 16);
  p->bcsr->copyToDevice(&p->hdr, &p->idx, &p->data);
  ck(cudaMalloc(&p->dB, (size_t)K * N * sizeof(half)), "cudaMalloc B");
  ck(cudaMalloc(&p->dC, (size_t)M * N * sizeof(float)), "cudaMalloc C");
  ck(cudaMemcpy(p->dB, p->B->data, (size_t)K * N * sizeof(half), cudaMemcpyHostToDevice), "copy B");
  return p;
}

// C = A B on the host over A's stored blocks, in double, against the device
// result at the reference harness's tolerance (nvbench_main.cu:357-364).
bool check(const Problem& p, const char* name) {
  std::vector<float> got((size_t)p.M * p.N);
  ck(cudaMemcpy(got.data(), p.dC, got.size() * sizeof(float), cudaMemcpyDeviceToHost), "copy C");
  const BCSRMatrix& a = *p.bcsr;
  const int bR = a.blockSizeRow;
  std::vector<double> ref((size_t)p.M * p.N, 0.0);
  for (int br = 0; br < a.blockRows; ++br)
    for (int k = a.hdr[br]; k < a.hdr[br + 1]; ++k)
      for (int x = 0; x < bR; ++x)
        for (int y = 0; y < 16; ++y) {
          const double v = __half2float(a.data[(size_t)k * bR * 16 + x * 16 + y]);
          if (v == 0.0) continue;
          const half* brow = p.B->data + (size_t)(a.idx[k] * 16 + y) * p.N;
          double* crow = ref.data() + (size_t)(br * bR + x) * p.N;
          for (int j = 0; j < p.N; ++j) crow[j] += v * __half2float(brow[j]);
        }
  for (size_t i = 0; i < got.size(); ++i)
    if (!(std::fabs(got[i] - ref[i]) <= 1e-2)) {
      std::fprintf(stderr, "[%s] mismatch at index %zu: got %f expected %f (M=%d K=%d N=%d)\n", name, i, got[i],
                   ref[i], p.M, p.K, p.N);
      return false;
    }
  return true;
}

using Launcher = spmm_status (*)(const int*, const int*, const void*, const void*, float*, unsigned, unsigned,
                                 unsigned, void*);

// The body every shaped bench shares (the reference repeats it per kernel).
void run_bench(nvbench::state& state, Launcher launch_fn, int bR, const char* name) {
  const int M = static_cast<int>(state.get_int64("M"));
  const int K = static_cast<int>(state.get_int64("K"));
  const int N = static_cast<int>(state.get_int64("N"));
  const double spars = state.get_int64("SPARS") / 100.0;
  const std::string pattern = kPatterns.at(state.get_int64("PAT") % kPatterns.size());
  if (M % bR || K % 16 || N % 8) {
    state.skip("M must be a multiple of the block height, K of 16, N of 8");
    return;
  }
  auto p = make_problem(M, K, N, spars, pattern, bR);
  state.add_element_count(static_cast<size_t>(M) * N);
  spmm_status st = SPMM_OK;
  state.exec(nvbench::exec_tag::timer, [&](nvbench::launch& launch, auto& timer) {
    cudaMemsetAsync(p->dC, 0, static_cast<size_t>(M) * N * sizeof(float), launch.get_stream());
    timer.start();
    st = launch_fn(p->hdr, p->idx, p->data, p->dB, p->dC, static_cast<unsigned>(M), static_cast<unsigned>(N),
                   static_cast<unsigned>(K), launch.get_stream());
    timer.stop();
  });
  if (st != SPMM_OK) {
    std::fprintf(stderr, "[%s] launch failed: %s\n", name, spmm_last_error());
    std::exit(1);
  }
  if (spmm_device_error_check(state.get_cuda_stream()) != SPMM_OK) {
    std::fprintf(stderr, "[%s] %s\n", name, spmm_last_error());
    std::exit(1);
  }
  if (!check(*p, name)) std::exit(1);
  state.get_summary("nv/cold/time/gpu/min").remove_value("hide");
  state.get_summary("nv/cold/time/gpu/max").remove_value("hide");
}

// The Adaptive launchers take the reference's colBlocksPerRow (1, 2 or 3 by the
// aspect ratio M / K, nvbench_main.cu:1246-1252); the library ignores it.
using AdaptiveLauncher = spmm_status (*)(const int*, const int*, const void*, const void*, float*, unsigned,
                                         unsigned, unsigned, unsigned, void*);
template <AdaptiveLauncher L>
spmm_status adaptive_call(const int* h, const int* i, const void* d, const void* B, float* C, unsigned M, unsigned N,
                          unsigned K, void* s) {
  const double aspect = (double)M / (double)K;
  const unsigned col_blocks = aspect >= 4.0 ? 3u : aspect >= 2.0 ? 2u : 1u;
  return L(h, i, d, B, C, M, N, col_blocks, K, s);
}

#define SPMM_BENCH(NAME, BR, FN) \
  void bench_##NAME(nvbench::state& state) { run_bench(state, FN, BR, #NAME); }
SPMM_BENCH(sparseMatrixMulTensor, 16, sparseMatrixMulTensor_launch)
SPMM_BENCH(sparseMatrixMulTensor_v2, 16, sparseMatrixMulTensor_v2_launch)
SPMM_BENCH(sparseMatrixMulTensor_v3, 16, sparseMatrixMulTensor_v3_launch)
SPMM_BENCH(sparseMatrixMulTensor_v1_improved, 16, sparseMatrixMulTensor_v1_improved_launch)
SPMM_BENCH(sparseMatrixMulTensor32x16, 32, sparseMatrixMulTensor32x16_launch)
SPMM_BENCH(sparseMatrixMulTensor32x16_v2, 32, sparseMatrixMulTensor32x16_v2_launch)
SPMM_BENCH(sparseMatrixMulTensor32x16_shared, 32, sparseMatrixMulTensor32x16_shared_launch)
SPMM_BENCH(sparseMatrixMulTensor32x16_shared_vectorized, 32, sparseMatrixMulTensor32x16_shared_vectorized_launch)
SPMM_BENCH(sparseMatrixMulTensor32x16_v2_shared_vectorized, 32,
           sparseMatrixMulTensor32x16_v2_shared_vectorized_launch)
SPMM_BENCH(sparseMatrixMulTensor64x16, 64, sparseMatrixMulTensor64x16_launch)
SPMM_BENCH(sparseMatrixMulTensor64x16_v2, 64, sparseMatrixMulTensor64x16_v2_launch)
SPMM_BENCH(sparseMatrixMulTensorAdaptive, 16, adaptive_call<sparseMatrixMulTensorAdaptive_launch>)
SPMM_BENCH(sparseMatrixMulTensorAdaptive32x16, 32, adaptive_call<sparseMatrixMulTensorAdaptive32x16_launch>)
SPMM_BENCH(sparseMatrixMulTensorAdaptive64x16, 64, adaptive_call<sparseMatrixMulTensorAdaptive64x16_launch>)
#undef SPMM_BENCH

}  // namespace

// Registrations with the reference's axes (nvbench_main.cu:1417-1449: the
// M = 1024 / K = 256, M = 512 / K = 512 and M = 2048 / K = 256 sets, with the
// sparsities and patterns it sweeps per block shape).
#define SPMM_AXES(BENCH, NAME, PATS)                                                               \
  NVBENCH_BENCH(BENCH)                                                                             \
      .set_name(NAME)                                                                              \
      .add_int64_axis("N", {32, 64, 128})                                                          \
      .add_int64_axis("M", {512, 1024, 2048})                                                      \
      .add_int64_axis("K", {256, 512})                                                             \
      .add_int64_axis("SPARS", {60, 70, 80, 90})                                                   \
      .add_int64_axis("PAT", PATS)
SPMM_AXES(bench_sparseMatrixMulTensor, "sparseMatrixMulTensor", (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor_v2, "sparseMatrixMulTensor_v2", (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor_v3, "sparseMatrixMulTensor_v3", (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor_v1_improved, "sparseMatrixMulTensor_v1_improved",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor32x16, "sparseMatrixMulTensor32x16", (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor32x16_v2, "sparseMatrixMulTensor32x16_v2",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor32x16_shared, "sparseMatrixMulTensor32x16_shared",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor32x16_shared_vectorized, "sparseMatrixMulTensor32x16_shared_vectorized",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor32x16_v2_shared_vectorized, "sparseMatrixMulTensor32x16_v2_shared_vectorized",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor64x16, "sparseMatrixMulTensor64x16", (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensor64x16_v2, "sparseMatrixMulTensor64x16_v2",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensorAdaptive, "sparseMatrixMulTensorAdaptive_16x16",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensorAdaptive32x16, "sparseMatrixMulTensorAdaptive_32x16",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
SPMM_AXES(bench_sparseMatrixMulTensorAdaptive64x16, "sparseMatrixMulTensorAdaptive_64x16",
          (std::vector<nvbench::int64_t>{0, 1, 2, 3, 4, 5, 6}));
#undef SPMM_AXES

NVBENCH_MAIN
