// Launches the reference's own WMMA kernels (src/cuda_kernels.cu), compiled
// unmodified from the reference tree into _ref/ref_kernels.cubin, with the
// launch geometry of the reference harness (nvbench_main.cu). Test and baseline
// infrastructure only: it is how the GPU tests compare the library against the
// reference kernels on identical inputs, and how they are timed on the same GPU.
#include <cuda_runtime.h>
#include <cstring>
#include <map>
#include <string>

namespace {
std::map<std::string, cudaLibrary_t> g_libs;

struct Geometry { unsigned gx, gy, block, smem; bool adaptive; unsigned rows_per_cta; };

// Reference launch geometry per kernel (nvbench_main.cu:339-346, :393-402,
// :548-555, :648-655, :840-847, :1245-1262).
bool geometry(const std::string& k, unsigned M, unsigned N, Geometry* g) {
  auto cdiv = [](unsigned a, unsigned b) { return (a + b - 1) / b; };
  if (k == "sparseMatrixMulTensor") { *g = {cdiv(N, 16), cdiv(M, 16), 32, 0, false, 16}; return true; }
  if (k == "sparseMatrixMulTensor_v2") { *g = {cdiv(N, 32), cdiv(M, 16), 64, 0, false, 16}; return true; }
  if (k == "sparseMatrixMulTensor32x16") { *g = {cdiv(N, 32), cdiv(M, 32), 32, 0, false, 32}; return true; }
  if (k == "sparseMatrixMulTensor32x16_v2") { *g = {cdiv(N, 32), cdiv(M, 32), 64, 0, false, 32}; return true; }
  if (k == "sparseMatrixMulTensor64x16") { *g = {cdiv(N, 32), cdiv(M, 64), 32, 0, false, 64}; return true; }
  return false;
}

std::string mangled(const std::string& k) {
  return "_Z" + std::to_string(k.size()) + k + "PKiS0_PK6__halfS3_Pfjj";
}
}  // namespace

extern "C" int ref_wmma_launch(const char* cubin, const char* kernel, const int* hdr, const int* idx,
                               const void* data, const void* B, float* C, unsigned M, unsigned N,
                               void* stream) {
  Geometry g;
  if (!geometry(kernel, M, N, &g)) return -1;
  cudaLibrary_t lib;
  auto it = g_libs.find(cubin);
  if (it == g_libs.end()) {
    cudaError_t e = cudaLibraryLoadFromFile(&lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) return (int)e;
    g_libs[cubin] = lib;
  } else {
    lib = it->second;
  }
  cudaKernel_t k;
  cudaError_t e = cudaLibraryGetKernel(&k, lib, mangled(kernel).c_str());
  if (e != cudaSuccess) return (int)e;
  void* args[] = {&hdr, &idx, &data, &B, &C, &M, &N};
  e = cudaLaunchKernel(reinterpret_cast<const void*>(k), dim3(g.gx, g.gy), dim3(g.block), args, g.smem,
                       static_cast<cudaStream_t>(stream));
  return (int)e;
}
