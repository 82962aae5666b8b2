// The reference's host call sequence for one BCSR product, written against this
// library's C++ drop-in header (include/bcsr_spmm.hpp) and C ABI: generate A and
// B with mg::generate_matrix (seeds 123 and 456), build Matrix objects, convert A
// with the BCSRMatrix constructor, copyToDevice, launch the shaped launcher,
// copy C back (nvbench_main.cu:139-175 and :636-673; formats/BCSRMatrix.cu:106-132).
//
//   dropin_sequence M K N SPARSITY PATTERN BR OUT_PREFIX
//
// Writes OUT_PREFIX.c (M*N float32), OUT_PREFIX.hdr and OUT_PREFIX.idx (int32),
// for the test to compare with the oracle. Exit status 0 on success.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "bcsr_spmm.h"
#include "bcsr_spmm.hpp"

static bool write_file(const std::string& path, const void* p, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = std::fwrite(p, 1, bytes, f) == bytes;
  return std::fclose(f) == 0 && ok;
}

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: %s M K N SPARSITY PATTERN BR OUT_PREFIX\n", argv[0]);
    return 2;
  }
  const int M = std::atoi(argv[1]), K = std::atoi(argv[2]), N = std::atoi(argv[3]);
  const double sparsity = std::atof(argv[4]);
  const std::string pattern = argv[5], out = argv[7];
  const int bR = std::atoi(argv[6]);

  auto gA = mg::generate_matrix<float>(M, K, sparsity, pattern, bR, 123);
  auto gB = mg::generate_matrix<float>(K, N, 0.0, "random", bR, 456);
  Matrix A(M, K), B(K, N);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < K; ++j) A.data[(size_t)i * K + j] = __float2half(gA[i][j]);
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < N; ++j) B.data[(size_t)i * N + j] = __float2half(gB[i][j]);

  BCSRMatrix bcsr(A, bR, 16);
  int *hdr = nullptr, *idx = nullptr;
  half* data = nullptr;
  bcsr.copyToDevice(&hdr, &idx, &data);

  half* dB = nullptr;
  float* dC = nullptr;
  if (cudaMalloc(&dB, (size_t)K * N * sizeof(half)) != cudaSuccess ||
      cudaMalloc(&dC, (size_t)M * N * sizeof(float)) != cudaSuccess) {
    std::fprintf(stderr, "cudaMalloc failed\n");
    return 1;
  }
  cudaMemcpy(dB, B.data, (size_t)K * N * sizeof(half), cudaMemcpyHostToDevice);
  cudaMemset(dC, 0xff, (size_t)M * N * sizeof(float));   // NaN: every element must be written

  spmm_status st = bR == 16   ? sparseMatrixMulTensor_launch(hdr, idx, data, dB, dC, M, N, K, nullptr)
                   : bR == 32 ? sparseMatrixMulTensor32x16_launch(hdr, idx, data, dB, dC, M, N, K, nullptr)
                              : sparseMatrixMulTensor64x16_launch(hdr, idx, data, dB, dC, M, N, K, nullptr);
  if (st != SPMM_OK) {
    std::fprintf(stderr, "launch failed: %s\n", spmm_last_error());
    return 1;
  }
  if (spmm_device_error_check(nullptr) != SPMM_OK || cudaDeviceSynchronize() != cudaSuccess) {
    std::fprintf(stderr, "device error: %s\n", spmm_last_error());
    return 1;
  }
  std::vector<float> C((size_t)M * N);
  cudaMemcpy(C.data(), dC, C.size() * sizeof(float), cudaMemcpyDeviceToHost);
  const bool ok = write_file(out + ".c", C.data(), C.size() * sizeof(float)) &&
                  write_file(out + ".hdr", bcsr.hdr, (size_t)(bcsr.blockRows + 1) * sizeof(int)) &&
                  write_file(out + ".idx", bcsr.idx, (size_t)bcsr.hdr[bcsr.blockRows] * sizeof(int));
  cudaFree(hdr);
  cudaFree(idx);
  cudaFree(data);
  cudaFree(dB);
  cudaFree(dC);
  std::printf("nnzb=%d\n", bcsr.hdr[bcsr.blockRows]);
  return ok ? 0 : 1;
}
