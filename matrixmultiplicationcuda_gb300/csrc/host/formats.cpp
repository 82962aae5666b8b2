// Host formats: Matrix (+ .mat text I/O), CSRMatrix, BCSRMatrix, and the C-ABI
// wrappers the Python layer uses to reach them.
#include <cuda_runtime.h>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>
#include "../../../include/bcsr_spmm.hpp"
#include "host_internal.h"

namespace {

// Reads the whole file; throws when it cannot be opened.
std::string slurp(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + path + ": " + std::strerror(errno));
  std::string s;
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
  std::fclose(f);
  return s;
}

// Parses "rows cols v v v ..." (the .mat text format written by the
// reference's matrix_generator.py:110-122 and read by Matrix.cu:14-32).
// Returns false when the header is missing or fewer than rows*cols values follow.
bool parse_mat(const std::string& text, int* rows, int* cols, std::vector<float>* vals) {
  const char* p = text.c_str();
  char* end = nullptr;
  long r = std::strtol(p, &end, 10);
  if (end == p) return false;
  p = end;
  long c = std::strtol(p, &end, 10);
  if (end == p || r < 0 || c < 0) return false;
  p = end;
  *rows = (int)r;
  *cols = (int)c;
  if (!vals) return true;
  const size_t n = (size_t)r * (size_t)c;
  vals->resize(n);
  for (size_t i = 0; i < n; ++i) {
    float v = std::strtof(p, &end);
    if (end == p) return false;
    (*vals)[i] = v;
    p = end;
  }
  return true;
}

}  // namespace

// ---------------------------------------------------------------------------------
Matrix::Matrix(int rows_, int cols_) : rows(rows_), cols(cols_), nonZeros(0) {
  const size_t n = (size_t)rows * cols;
  data = static_cast<half*>(std::malloc(n * sizeof(half) + 16));
  std::memset(data, 0, n * sizeof(half));
}

Matrix::Matrix(const std::string& filename) {
  std::vector<float> v;
  if (!parse_mat(slurp(filename), &rows, &cols, &v))
    throw std::runtime_error("malformed .mat file: " + filename);
  const size_t n = (size_t)rows * cols;
  data = static_cast<half*>(std::malloc(n * sizeof(half) + 16));
  nonZeros = 0;
  for (size_t i = 0; i < n; ++i) {
    if (v[i] != 0.0f) nonZeros++;
    data[i] = __float2half(v[i]);
  }
}

Matrix::~Matrix() { std::free(data); }

void Matrix::print() const {
  std::cout << rows << ' ' << cols << "\n===\n";
  for (int i = 0; i < rows; i++) {
    for (int j = 0; j < cols; j++) std::cout << __half2float(data[(size_t)i * cols + j]) << " ";
    std::cout << "\n";
  }
}

static inline bool h_nonzero(half h) {
  unsigned short b;
  std::memcpy(&b, &h, 2);
  return (b & 0x7fffu) != 0;  // float(h) != 0: all but +0 / -0 (NaN counts)
}

float blockDensity(const Matrix& m, int i, int j, int bR, int bC) {
  int nz = 0;
  for (int x = i; x < i + bR; x++)
    for (int y = j; y < j + bC; y++)
      if (h_nonzero(m.data[(size_t)x * m.cols + y])) nz++;
  return (float)nz / (float)(bR * bC);
}

// ---------------------------------------------------------------------------------
CSRMatrix::CSRMatrix(const Matrix& m) {
  N = m.rows;
  hdr = static_cast<int*>(std::malloc((m.rows + 1) * sizeof(int)));
  hdr[0] = 0;
  for (int i = 0; i < m.rows; i++) {
    hdr[i + 1] = hdr[i];
    for (int j = 0; j < m.cols; j++)
      if (h_nonzero(m.data[(size_t)i * m.cols + j])) hdr[i + 1]++;
  }
  idx = static_cast<int*>(std::malloc((size_t)hdr[m.rows] * sizeof(int) + 4));
  data = static_cast<half*>(std::malloc((size_t)hdr[m.rows] * sizeof(half) + 4));
  size_t k = 0;
  for (size_t i = 0; i < (size_t)m.rows * m.cols; i++)
    if (h_nonzero(m.data[i])) {
      idx[k] = (int)(i % (size_t)m.cols);
      data[k] = m.data[i];
      k++;
    }
}

CSRMatrix::~CSRMatrix() {
  std::free(hdr);
  std::free(idx);
  std::free(data);
}

static void dev_copy(void** dst, const void* src, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(dst, bytes ? bytes : 16);
  if (e == cudaSuccess && bytes) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess)
    throw std::runtime_error(std::string(what) + " CUDA error: " + cudaGetErrorString(e));
}

void CSRMatrix::copyToDevice(int** gpuHdr, int** gpuIdx, half** gpuData) const {
  dev_copy(reinterpret_cast<void**>(gpuData), data, (size_t)hdr[N] * sizeof(half), "CSRMatrix::copyToDevice");
  dev_copy(reinterpret_cast<void**>(gpuHdr), hdr, (size_t)(N + 1) * sizeof(int), "CSRMatrix::copyToDevice");
  dev_copy(reinterpret_cast<void**>(gpuIdx), idx, (size_t)hdr[N] * sizeof(int), "CSRMatrix::copyToDevice");
}

// ---------------------------------------------------------------------------------
BCSRMatrix::BCSRMatrix(const Matrix& m, int bR, int bC) : blockSizeRow(bR), blockSizeCol(bC) {
  if (bR < 16 || bC < 16)
    throw std::invalid_argument("Block sizes must be at least 16x16 for WMMA compatibility. Got " +
                                std::to_string(bR) + "x" + std::to_string(bC));
  if (bR % 16 != 0 || bC % 16 != 0)
    throw std::invalid_argument("Block sizes must be multiples of 16 for WMMA alignment. Got " +
                                std::to_string(bR) + "x" + std::to_string(bC));
  blockRows = m.rows / bR;
  blockCols = m.cols / bC;
  // One scan marks the kept blocks; a second pass compacts them.
  std::vector<unsigned char> keep((size_t)blockRows * blockCols, 0);
  hdr = static_cast<int*>(std::malloc((size_t)(blockRows + 1) * sizeof(int)));
  hdr[0] = 0;
  for (int br = 0; br < blockRows; ++br) {
    int cnt = 0;
    for (int bc = 0; bc < blockCols; ++bc) {
      bool nz = false;
      for (int x = 0; x < bR && !nz; ++x) {
        const half* row = m.data + (size_t)(br * bR + x) * m.cols + (size_t)bc * bC;
        for (int y = 0; y < bC; ++y)
          if (h_nonzero(row[y])) { nz = true; break; }
      }
      keep[(size_t)br * blockCols + bc] = nz;
      cnt += nz;
    }
    hdr[br + 1] = hdr[br] + cnt;
  }
  const size_t nnzb = (size_t)hdr[blockRows];
  idx = static_cast<int*>(std::malloc(nnzb * sizeof(int) + 4));
  data = static_cast<half*>(std::malloc(nnzb * (size_t)bR * bC * sizeof(half) + 16));
  size_t k = 0;
  for (int br = 0; br < blockRows; ++br)
    for (int bc = 0; bc < blockCols; ++bc) {
      if (!keep[(size_t)br * blockCols + bc]) continue;
      idx[k] = bc;
      for (int x = 0; x < bR; ++x)
        std::memcpy(data + k * bR * bC + (size_t)x * bC,
                    m.data + (size_t)(br * bR + x) * m.cols + (size_t)bc * bC, bC * sizeof(half));
      nonZeros += bR * bC;
      ++k;
    }
}

BCSRMatrix::~BCSRMatrix() {
  std::free(hdr);
  std::free(idx);
  std::free(data);
}

void BCSRMatrix::print() const {
  std::cout << "Block size: " << blockSizeRow << "x" << blockSizeCol << std::endl;
  std::cout << "hdr:\n\t";
  for (int i = 0; i <= blockRows; i++) std::cout << hdr[i] << " ";
  std::cout << "\nidx:\n\t";
  for (int i = 0; i < hdr[blockRows]; i++) std::cout << idx[i] << " ";
  std::cout << "\ndata:\n";
  for (int i = 0; i < hdr[blockRows]; i++) {
    std::cout << "=== Block " << i << " ===\n";
    for (int j = 0; j < blockSizeRow; j++) {
      std::cout << '\t';
      for (int k = 0; k < blockSizeCol; k++)
        std::cout << __half2float(data[(size_t)i * blockSizeRow * blockSizeCol + j * blockSizeCol + k]) << " ";
      std::cout << '\n';
    }
  }
}

void BCSRMatrix::copyToDevice(int** gpuHdr, int** gpuIdx, half** gpuData) const {
  const size_t nnzb = (size_t)hdr[blockRows];
  dev_copy(reinterpret_cast<void**>(gpuHdr), hdr, (size_t)(blockRows + 1) * sizeof(int), "BCSRMatrix::copyToDevice");
  dev_copy(reinterpret_cast<void**>(gpuIdx), idx, nnzb * sizeof(int), "BCSRMatrix::copyToDevice");
  dev_copy(reinterpret_cast<void**>(gpuData), data, nnzb * blockSizeRow * blockSizeCol * sizeof(half),
           "BCSRMatrix::copyToDevice");
}

// ---------------------------------------------------------------------------------
// Splits the blocks by density into two zero-initialised copies of the matrix,
// as the reference does, then builds the two formats from them.
HCSRMatrix::HCSRMatrix(const Matrix& m, float threshold) {
  if (m.rows % 16 || m.cols % 16)
    throw std::invalid_argument("HCSRMatrix needs rows and columns that are multiples of 16");
  Matrix dense_part(m.rows, m.cols), sparse_part(m.rows, m.cols);
  for (int i = 0; i < m.rows; i += 16)
    for (int j = 0; j < m.cols; j += 16) {
      Matrix& dst = blockDensity(m, i, j, 16, 16) >= threshold ? dense_part : sparse_part;
      for (int x = i; x < i + 16; ++x)
        std::memcpy(dst.data + (size_t)x * m.cols + j, m.data + (size_t)x * m.cols + j, 16 * sizeof(half));
    }
  bcsr = new BCSRMatrix(dense_part, 16, 16);
  csr = new CSRMatrix(sparse_part);
}

HCSRMatrix::~HCSRMatrix() {
  delete bcsr;
  delete csr;
}

// ---------------------------------------------------------------------------------
// C ABI over the classes (used by the Python layer and by callers without C++).
extern "C" {

spmm_status spmm_mat_read_header(const char* path, int* rows, int* cols) {
  try {
    std::string t = slurp(path);
    if (!parse_mat(t, rows, cols, nullptr)) return spmm::host_fail(SPMM_ERR_INVALID_ARG, "malformed .mat header");
    return SPMM_OK;
  } catch (const std::exception& e) {
    return spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
  }
}

spmm_status spmm_mat_load(const char* path, void* out_half, size_t capacity, int* rows, int* cols,
                          int* nonZeros) {
  try {
    Matrix m{std::string(path)};
    const size_t n = (size_t)m.rows * m.cols;
    *rows = m.rows;
    *cols = m.cols;
    *nonZeros = m.nonZeros;
    if (n > capacity) return spmm::host_fail(SPMM_ERR_INVALID_ARG, "output buffer too small");
    std::memcpy(out_half, m.data, n * sizeof(half));
    return SPMM_OK;
  } catch (const std::exception& e) {
    return spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
  }
}

spmm_status spmm_mat_save(const char* path, const float* vals, int rows, int cols) {
  FILE* f = std::fopen(path, "w");
  if (!f) return spmm::host_fail(SPMM_ERR_INVALID_ARG, std::string("cannot write ") + path);
  std::fprintf(f, "%d %d\n", rows, cols);
  for (int i = 0; i < rows; ++i) {
    for (int j = 0; j < cols; ++j) std::fprintf(f, j ? " %.9g" : "%.9g", vals[(size_t)i * cols + j]);
    std::fputc('\n', f);
  }
  std::fclose(f);
  return SPMM_OK;
}

// BCSRMatrix on the host: returns nnzb, fills the arrays when non-null.
long long spmm_host_dense_to_bcsr(const void* A_half, int rows, int cols, int bR, int bC,
                                  int* hdr, int* idx, void* vals) {
  try {
    Matrix m(rows, cols);
    std::memcpy(m.data, A_half, (size_t)rows * cols * sizeof(half));
    BCSRMatrix b(m, bR, bC);
    const long long nnzb = b.hdr[b.blockRows];
    if (hdr) std::memcpy(hdr, b.hdr, sizeof(int) * (b.blockRows + 1));
    if (idx) std::memcpy(idx, b.idx, sizeof(int) * nnzb);
    if (vals) std::memcpy(vals, b.data, sizeof(half) * nnzb * bR * bC);
    return nnzb;
  } catch (const std::exception& e) {
    spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
    return -1;
  }
}

// HCSRMatrix on the host: the sizes of both parts, and their arrays where the
// output pointers are non-null. Returns 0, or -1 on bad arguments.
int spmm_host_dense_to_hcsr(const void* A_half, int rows, int cols, float threshold, long long* nnzb,
                            long long* nnz, int* bhdr, int* bidx, void* bvals, int* chdr, int* cidx, void* cvals) {
  try {
    if (!A_half || !nnzb || !nnz || rows < 0 || cols < 0) throw std::invalid_argument("bad arguments");
    Matrix m(rows, cols);
    std::memcpy(m.data, A_half, (size_t)rows * cols * sizeof(half));
    HCSRMatrix h(m, threshold);
    *nnzb = h.bcsr->hdr[h.bcsr->blockRows];
    *nnz = h.csr->hdr[rows];
    if (bhdr) std::memcpy(bhdr, h.bcsr->hdr, sizeof(int) * (h.bcsr->blockRows + 1));
    if (bidx) std::memcpy(bidx, h.bcsr->idx, sizeof(int) * *nnzb);
    if (bvals) std::memcpy(bvals, h.bcsr->data, sizeof(half) * *nnzb * 256);
    if (chdr) std::memcpy(chdr, h.csr->hdr, sizeof(int) * (rows + 1));
    if (cidx) std::memcpy(cidx, h.csr->idx, sizeof(int) * *nnz);
    if (cvals) std::memcpy(cvals, h.csr->data, sizeof(half) * *nnz);
    return 0;
  } catch (const std::exception& e) {
    spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
    return -1;
  }
}

// CSRMatrix on the host (column index fixed to i % cols): returns nnz.
long long spmm_host_dense_to_csr(const void* A_half, int rows, int cols, int* hdr, int* idx,
                                 void* vals) {
  Matrix m(rows, cols);
  std::memcpy(m.data, A_half, (size_t)rows * cols * sizeof(half));
  CSRMatrix c(m);
  const long long nnz = c.hdr[rows];
  if (hdr) std::memcpy(hdr, c.hdr, sizeof(int) * (rows + 1));
  if (idx) std::memcpy(idx, c.idx, sizeof(int) * nnz);
  if (vals) std::memcpy(vals, c.data, sizeof(half) * nnz);
  return nnz;
}

}  // extern "C"
