// bcsr_spmm.hpp -- C++ host API that mirrors the reference's host classes, so
// code written against Matrix / CSRMatrix / BCSRMatrix / mg::generate_matrix of
// hosseinal/MatrixMultiplicationCUDA compiles against this library unchanged.
//
//   Matrix       <- Matrix.cuh:12-23, Matrix.cu:6-46
//   CSRMatrix    <- formats/CSRMatrix.cuh:11-21, formats/CSRMatrix.cu:13-63
//   BCSRMatrix   <- formats/BCSRMatrix.cuh:9-26, formats/BCSRMatrix.cu:22-132
//   mg::generate_matrix <- matrix_generator.h:28-34, matrix_generator.cpp:28-140
//
// Differences, all deliberate:
//   * Matrix(path) parses the .mat text itself instead of redirecting stdin
//     (Matrix.cu:18 calls freopen(path, "r", stdin)); a missing file throws.
//   * CSRMatrix stores the column index (i % cols); the reference stores
//     i % rows (formats/CSRMatrix.cu:32), which is only right for square A.
//   * copyToDevice reports failures by throwing std::runtime_error instead of
//     assert() (formats/BCSRMatrix.cu:15-19); the caller owns and frees the
//     returned device arrays, as in the reference.
#pragma once
#include <cuda_fp16.h>
#include <stdexcept>
#include <string>
#include <vector>
#include "bcsr_spmm.h"

class Matrix {
 public:
  half* data = nullptr;
  int rows = 0;
  int cols = 0;
  int nonZeros = 0;
  Matrix(int rows, int cols);
  explicit Matrix(const std::string& filename);
  ~Matrix();
  Matrix(const Matrix&) = delete;
  Matrix& operator=(const Matrix&) = delete;
  void print() const;
};

class CSRMatrix {
 public:
  int N = 0;                 // rows
  int *hdr = nullptr, *idx = nullptr;
  half* data = nullptr;
  explicit CSRMatrix(const Matrix& matrix);
  ~CSRMatrix();
  CSRMatrix(const CSRMatrix&) = delete;
  CSRMatrix& operator=(const CSRMatrix&) = delete;
  void copyToDevice(int** gpuHdr, int** gpuIdx, half** gpuData) const;
};

class BCSRMatrix {
 public:
  int* hdr = nullptr;
  int* idx = nullptr;
  half* data = nullptr;
  int blockRows = 0;
  int blockCols = 0;
  int nonZeros = 0;          // stored elements (kept blocks x bR x bC), as the reference counts
  int blockSizeRow = 0;
  int blockSizeCol = 0;
  explicit BCSRMatrix(const Matrix& matrix, int blockSizeRow = 16, int blockSizeCol = 16);
  ~BCSRMatrix();
  BCSRMatrix(const BCSRMatrix&) = delete;
  BCSRMatrix& operator=(const BCSRMatrix&) = delete;
  void print() const;
  void copyToDevice(int** gpuHdr, int** gpuIdx, half** gpuData) const;
};

// HCSRMatrix(matrix, threshold) (formats/HCSRMatrix.cpp:10-36): the 16x16
// blocks whose density (nonzero elements / 256) is >= threshold form a 16x16
// BCSR part, every other element a CSR part. spmm_hcsr_mm multiplies both
// parts in one launch.
class HCSRMatrix {
 public:
  BCSRMatrix* bcsr = nullptr;
  CSRMatrix* csr = nullptr;
  HCSRMatrix(const Matrix& matrix, float threshold);
  ~HCSRMatrix();
  HCSRMatrix(const HCSRMatrix&) = delete;
  HCSRMatrix& operator=(const HCSRMatrix&) = delete;
};

// blockDensity (miscutil.cpp:76-87): fraction of elements of the bR x bC block
// at (i, j) whose value compares != 0.
float blockDensity(const Matrix& matrix, int i, int j, int blockSizeRow = 16, int blockSizeCol = 16);

namespace mg {
template <typename T>
using Matrix = std::vector<std::vector<T>>;
// Same patterns, RNG stream and output as the reference generator for T = float.
template <typename T>
Matrix<T> generate_matrix(int num_rows, int num_cols, double sparsity = 0.7,
                          const std::string& pattern = "random", int blocksize = 16,
                          unsigned int seed = 123u);
}  // namespace mg
