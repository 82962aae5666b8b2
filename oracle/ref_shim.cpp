// C entry points over the reference's own host code (generator, Matrix,
// BCSRMatrix, CSRMatrix, miscutil), compiled from the reference tree by
// `make ref`. Used only to pin the oracle restatement and to write the golden
// fixtures; it never ships and never runs on the GPU host (the reference tree
// is not there).
#include <cstdint>
#include <cstring>
#include <vector>
#include <string>
#include <cuda_fp16.h>
#include "Matrix.cuh"
#include "formats/BCSRMatrix.cuh"
#include "formats/CSRMatrix.cuh"
#include "formats/HCSRMatrix.h"
#include "miscutil.h"
#include "matrix_generator.h"

extern const int BLOCK_SIZE = 16;

extern "C" {

// mg::generate_matrix<float> straight from the reference.
int ref_generate_matrix(int rows, int cols, double sparsity, const char* pattern,
                        int blocksize, unsigned seed, float* out) {
  try {
    auto m = mg::generate_matrix<float>(rows, cols, sparsity, std::string(pattern), blocksize, seed);
    for (int i = 0; i < rows; ++i) std::memcpy(out + (size_t)i * cols, m[i].data(), sizeof(float) * cols);
    return 0;
  } catch (...) {
    return -1;
  }
}

// The reference's float -> half conversion path (fill_Matrix_from_generated uses __float2half).
void ref_f32_to_f16(const float* in, uint16_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) { half h = __float2half(in[i]); std::memcpy(out + i, &h, 2); }
}

// BCSRMatrix(matrix, bR, bC): returns nnzb and, when the output pointers are
// non-null, copies hdr/idx/data out. Returns -1 when the ctor throws.
long long ref_bcsr(const uint16_t* A, int rows, int cols, int bR, int bC,
                   int* hdr, int* idx, uint16_t* data, int* nonZeros) {
  Matrix m(rows, cols);
  std::memcpy(m.data, A, sizeof(uint16_t) * (size_t)rows * cols);
  try {
    BCSRMatrix b(m, bR, bC);
    long long nnzb = b.hdr[b.blockRows];
    if (hdr) std::memcpy(hdr, b.hdr, sizeof(int) * (b.blockRows + 1));
    if (idx) std::memcpy(idx, b.idx, sizeof(int) * nnzb);
    if (data) std::memcpy(data, b.data, sizeof(uint16_t) * nnzb * bR * bC);
    if (nonZeros) *nonZeros = b.nonZeros;
    return nnzb;
  } catch (...) {
    return -1;
  }
}

// HCSRMatrix(matrix, threshold): sizes of both parts, and their arrays when the
// output pointers are non-null (the CSR part's idx as the reference stores it).
int ref_hcsr(const uint16_t* A, int rows, int cols, float threshold, long long* nnzb, long long* nnz,
             int* bhdr, int* bidx, uint16_t* bdata, int* chdr, int* cidx, uint16_t* cdata) {
  Matrix m(rows, cols);
  std::memcpy(m.data, A, sizeof(uint16_t) * (size_t)rows * cols);
  HCSRMatrix h(m, threshold);
  *nnzb = h.bcsr->hdr[h.bcsr->blockRows];
  *nnz = h.csr->hdr[rows];
  if (bhdr) std::memcpy(bhdr, h.bcsr->hdr, sizeof(int) * (h.bcsr->blockRows + 1));
  if (bidx) std::memcpy(bidx, h.bcsr->idx, sizeof(int) * *nnzb);
  if (bdata) std::memcpy(bdata, h.bcsr->data, sizeof(uint16_t) * *nnzb * 256);
  if (chdr) std::memcpy(chdr, h.csr->hdr, sizeof(int) * (rows + 1));
  if (cidx) std::memcpy(cidx, h.csr->idx, sizeof(int) * *nnz);
  if (cdata) std::memcpy(cdata, h.csr->data, sizeof(uint16_t) * *nnz);
  delete h.bcsr;
  delete h.csr;
  return 0;
}

float ref_block_density(const uint16_t* A, int rows, int cols, int i, int j, int bR, int bC) {
  Matrix m(rows, cols);
  std::memcpy(m.data, A, sizeof(uint16_t) * (size_t)rows * cols);
  return blockDensity(m, i, j, bR, bC);
}

// Matrix(".mat path"): rows, cols, nonZeros and the half data (caller sizes `out`).
int ref_load_mat(const char* path, int* rows, int* cols, int* nonZeros, uint16_t* out, size_t cap) {
  Matrix m{std::string(path)};
  *rows = m.rows; *cols = m.cols; *nonZeros = m.nonZeros;
  size_t n = (size_t)m.rows * m.cols;
  if (out && n <= cap) std::memcpy(out, m.data, n * 2);
  return 0;
}

float ref_maxdiff(const float* A, const float* B, unsigned n) { return maxdiff(A, B, n); }
float ref_avgrelerr(const float* A, const float* B, unsigned n) { return avgrelerr(A, B, n); }
double ref_rmse(const float* A, const float* B, unsigned n) { return rmse(A, B, n); }

}
