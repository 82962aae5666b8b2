// File formats beside the reference's .mat text format:
//
// * Matrix Market (.mtx), the format the reference's generator writes through
//   scipy's mmwrite (matrix_generator.py:100-108) but never reads back. The
//   "matrix coordinate" (real, integer or pattern; general, symmetric or
//   skew-symmetric) and "matrix array" (real or integer, general) variants
//   load into a dense fp16 matrix -- as Matrix(".mat") does -- or straight into
//   BCSR without a dense copy (for matrices too large to hold densely).
//   Entries listed twice are summed. A BCSR block is kept when any of its
//   values, rounded to fp16, is nonzero: the rule of the BCSR constructor.
// * A binary BCSR file ("SPMMBCS1"): the arrays as they lie in memory, for
//   matrices that the text formats make impractically slow.
#include <cuda_fp16.h>
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
#include "../../../include/bcsr_spmm_host.h"
#include "host_internal.h"

namespace {

struct MtxHeader {
  bool coordinate = true, pattern = false, symmetric = false, skew = false;
  long long rows = 0, cols = 0, entries = 0;
};

struct Entry {
  long long r, c;
  double v;
};

std::string lower(std::string s) {
  for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

// Reads a Matrix Market file: the header and every entry (0-based, symmetric
// entries mirrored). Throws std::runtime_error on anything malformed.
MtxHeader read_mtx(const char* path, std::vector<Entry>* out) {
  FILE* f = std::fopen(path, "r");
  if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  struct Closer {
    FILE* f;
    ~Closer() { std::fclose(f); }
  } closer{f};
  char line[4096];
  if (!std::fgets(line, sizeof line, f)) throw std::runtime_error("empty file");
  char banner[64], object[64], format[64], field[64], sym[64];
  if (std::sscanf(line, "%63s %63s %63s %63s %63s", banner, object, format, field, sym) != 5 ||
      lower(banner) != "%%matrixmarket" || lower(object) != "matrix")
    throw std::runtime_error("not a Matrix Market matrix file");
  MtxHeader h;
  const std::string fmt = lower(format), fld = lower(field), sy = lower(sym);
  if (fmt == "coordinate") h.coordinate = true;
  else if (fmt == "array") h.coordinate = false;
  else throw std::runtime_error("unknown format " + fmt);
  if (fld == "pattern") h.pattern = true;
  else if (fld != "real" && fld != "integer" && fld != "double") throw std::runtime_error("unsupported field " + fld);
  if (sy == "symmetric") h.symmetric = true;
  else if (sy == "skew-symmetric") h.skew = true;
  else if (sy != "general") throw std::runtime_error("unsupported symmetry " + sy);
  if (!h.coordinate && (h.pattern || h.symmetric || h.skew))
    throw std::runtime_error("array format: only real / integer general matrices");
  // size line (after comments)
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == '%') continue;
    if (h.coordinate) {
      if (std::sscanf(line, "%lld %lld %lld", &h.rows, &h.cols, &h.entries) != 3)
        throw std::runtime_error("bad size line");
    } else {
      if (std::sscanf(line, "%lld %lld", &h.rows, &h.cols) != 2) throw std::runtime_error("bad size line");
      h.entries = h.rows * h.cols;
    }
    break;
  }
  if (h.rows <= 0 || h.cols <= 0 || h.rows > (1LL << 31) || h.cols > (1LL << 31) || h.entries < 0)
    throw std::runtime_error("bad matrix size");
  if (!out) return h;
  out->reserve((size_t)h.entries * ((h.symmetric || h.skew) ? 2 : 1));
  for (long long k = 0; k < h.entries; ++k) {
    Entry e{0, 0, 1.0};
    if (h.coordinate) {
      int got = h.pattern ? std::fscanf(f, "%lld %lld", &e.r, &e.c) : std::fscanf(f, "%lld %lld %lf", &e.r, &e.c, &e.v);
      if (got != (h.pattern ? 2 : 3)) throw std::runtime_error("truncated entry list");
      e.r -= 1;
      e.c -= 1;
      if (e.r < 0 || e.r >= h.rows || e.c < 0 || e.c >= h.cols) throw std::runtime_error("entry index out of range");
    } else {
      if (std::fscanf(f, "%lf", &e.v) != 1) throw std::runtime_error("truncated value list");
      e.r = k % h.rows;   // column-major
      e.c = k / h.rows;
    }
    out->push_back(e);
    if ((h.symmetric || h.skew) && e.r != e.c) out->push_back(Entry{e.c, e.r, h.skew ? -e.v : e.v});
  }
  return h;
}

bool half_nonzero(float v) {
  const __half h = __float2half(v);
  uint16_t b;
  std::memcpy(&b, &h, 2);
  return (b & 0x7fffu) != 0;
}

// Sums duplicate entries: (row, col) -> value, ordered row-major.
std::vector<Entry> sum_duplicates(std::vector<Entry> es, long long cols) {
  std::sort(es.begin(), es.end(), [cols](const Entry& a, const Entry& b) { return a.r * cols + a.c < b.r * cols + b.c; });
  std::vector<Entry> out;
  for (const Entry& e : es) {
    if (!out.empty() && out.back().r == e.r && out.back().c == e.c) out.back().v += e.v;
    else out.push_back(e);
  }
  return out;
}

constexpr char kMagic[8] = {'S', 'P', 'M', 'M', 'B', 'C', 'S', '1'};

size_t elem_size(int dtype) { return dtype == SPMM_E4M3 ? 1 : 2; }

}  // namespace

extern "C" {

spmm_status spmm_mtx_read_header(const char* path, int* rows, int* cols, long long* entries) {
  try {
    MtxHeader h = read_mtx(path, nullptr);
    if (rows) *rows = (int)h.rows;
    if (cols) *cols = (int)h.cols;
    if (entries) *entries = h.entries;
    return SPMM_OK;
  } catch (const std::exception& e) {
    return spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
  }
}

spmm_status spmm_mtx_load(const char* path, void* out_half, size_t capacity, int* rows, int* cols, int* nonZeros) {
  try {
    std::vector<Entry> es;
    MtxHeader h = read_mtx(path, &es);
    *rows = (int)h.rows;
    *cols = (int)h.cols;
    const size_t n = (size_t)h.rows * (size_t)h.cols;
    if (!out_half || n > capacity) return spmm::host_fail(SPMM_ERR_INVALID_ARG, "output buffer too small");
    std::vector<float> dense(n, 0.f);
    for (const Entry& e : es) dense[(size_t)e.r * h.cols + e.c] += (float)e.v;
    __half* out = static_cast<__half*>(out_half);
    int nz = 0;
    for (size_t i = 0; i < n; ++i) {
      out[i] = __float2half(dense[i]);
      if (dense[i] != 0.0f) ++nz;
    }
    if (nonZeros) *nonZeros = nz;
    return SPMM_OK;
  } catch (const std::exception& e) {
    return spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
  }
}

spmm_status spmm_mtx_load_bcsr(const char* path, int bR, int bC, int* rows, int* cols, int* row_ptr,
                               long long* nnzb, int* col_idx, void* vals, long long capacity_blocks) {
  try {
    if (bR < 16 || bC < 16 || bR % 16 || bC % 16) throw std::runtime_error("block sizes must be multiples of 16");
    std::vector<Entry> es;
    MtxHeader h = read_mtx(path, &es);
    es = sum_duplicates(std::move(es), h.cols);
    *rows = (int)h.rows;
    *cols = (int)h.cols;
    const long long MB = h.rows / bR, KB = h.cols / bC;
    // kept blocks: any entry inside the whole-block area whose fp16 value is nonzero
    std::map<long long, int> blocks;   // block id -> position, row-major
    for (const Entry& e : es) {
      if (e.r >= MB * bR || e.c >= KB * bC || !half_nonzero((float)e.v)) continue;
      blocks.emplace((e.r / bR) * KB + e.c / bC, 0);
    }
    *nnzb = (long long)blocks.size();
    if (row_ptr) {
      std::vector<int> cnt(MB + 1, 0);
      for (const auto& b : blocks) cnt[b.first / KB + 1]++;
      for (long long i = 0; i < MB; ++i) cnt[i + 1] += cnt[i];
      std::memcpy(row_ptr, cnt.data(), sizeof(int) * (MB + 1));
    }
    if (!col_idx || !vals || capacity_blocks < *nnzb) return SPMM_OK;
    int k = 0;
    for (auto& b : blocks) {
      b.second = k;
      col_idx[k++] = (int)(b.first % KB);
    }
    __half* v = static_cast<__half*>(vals);
    const __half zero = __float2half(0.f);
    std::fill(v, v + (size_t)*nnzb * bR * bC, zero);
    for (const Entry& e : es) {
      if (e.r >= MB * bR || e.c >= KB * bC) continue;
      auto it = blocks.find((e.r / bR) * KB + e.c / bC);
      if (it == blocks.end()) continue;
      v[(size_t)it->second * bR * bC + (e.r % bR) * bC + (e.c % bC)] = __float2half((float)e.v);
    }
    return SPMM_OK;
  } catch (const std::exception& e) {
    return spmm::host_fail(SPMM_ERR_INVALID_ARG, e.what());
  }
}

spmm_status spmm_mtx_save(const char* path, const float* vals, int rows, int cols) {
  if (!path || !vals || rows < 0 || cols < 0) return spmm::host_fail(SPMM_ERR_INVALID_ARG, "bad arguments");
  long long nnz = 0;
  for (size_t i = 0; i < (size_t)rows * cols; ++i) nnz += vals[i] != 0.0f;
  FILE* f = std::fopen(path, "w");
  if (!f) return spmm::host_fail(SPMM_ERR_INVALID_ARG, std::string("cannot write ") + path);
  std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n%d %d %lld\n", rows, cols, nnz);
  for (int i = 0; i < rows; ++i)
    for (int j = 0; j < cols; ++j) {
      const float v = vals[(size_t)i * cols + j];
      if (v != 0.0f) std::fprintf(f, "%d %d %.9g\n", i + 1, j + 1, v);
    }
  std::fclose(f);
  return SPMM_OK;
}

spmm_status spmm_bcsr_save(const char* path, int M, int K, int bR, int bC, int dtype, long long nnzb,
                           const int* row_ptr, const int* col_idx, const void* vals, const void* vals_lo,
                           const float* scales) {
  if (!path || M < 0 || K < 0 || bR <= 0 || bC <= 0 || M % bR || K % bC || dtype < 0 || dtype > 3 || nnzb < 0 ||
      !row_ptr || (nnzb && (!col_idx || !vals)) || (dtype == SPMM_F16_SPLIT && nnzb && !vals_lo) ||
      (dtype == SPMM_E4M3 && nnzb && !scales))
    return spmm::host_fail(SPMM_ERR_INVALID_ARG, "bad BCSR arguments");
  FILE* f = std::fopen(path, "wb");
  if (!f) return spmm::host_fail(SPMM_ERR_INVALID_ARG, std::string("cannot write ") + path);
  const int32_t hdr[6] = {M, K, bR, bC, dtype, 0};
  const size_t nv = (size_t)nnzb * bR * bC;
  bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof hdr, 1, f) == 1 &&
            std::fwrite(&nnzb, sizeof nnzb, 1, f) == 1 &&
            std::fwrite(row_ptr, sizeof(int), M / bR + 1, f) == (size_t)(M / bR + 1) &&
            (!nnzb || std::fwrite(col_idx, sizeof(int), nnzb, f) == (size_t)nnzb) &&
            (!nnzb || std::fwrite(vals, elem_size(dtype), nv, f) == nv);
  if (ok && nnzb && dtype == SPMM_F16_SPLIT) ok = std::fwrite(vals_lo, 2, nv, f) == nv;
  if (ok && nnzb && dtype == SPMM_E4M3) ok = std::fwrite(scales, sizeof(float), nnzb, f) == (size_t)nnzb;
  ok = std::fclose(f) == 0 && ok;
  return ok ? SPMM_OK : spmm::host_fail(SPMM_ERR_INVALID_ARG, std::string("write failed: ") + path);
}

spmm_status spmm_bcsr_load(const char* path, int* M, int* K, int* bR, int* bC, int* dtype, long long* nnzb,
                           int* row_ptr, int* col_idx, void* vals, void* vals_lo, float* scales,
                           long long capacity_blocks) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return spmm::host_fail(SPMM_ERR_INVALID_ARG, std::string("cannot open ") + path);
  char magic[8];
  int32_t hdr[6];
  long long n = 0;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0 &&
            std::fread(hdr, sizeof hdr, 1, f) == 1 && std::fread(&n, sizeof n, 1, f) == 1 && hdr[0] >= 0 &&
            hdr[1] >= 0 && hdr[2] > 0 && hdr[3] > 0 && hdr[0] % hdr[2] == 0 && hdr[1] % hdr[3] == 0 &&
            hdr[4] >= 0 && hdr[4] <= 3 && n >= 0;
  if (!ok) {
    std::fclose(f);
    return spmm::host_fail(SPMM_ERR_INVALID_ARG, std::string("not a BCSR file: ") + path);
  }
  *M = hdr[0];
  *K = hdr[1];
  *bR = hdr[2];
  *bC = hdr[3];
  *dtype = hdr[4];
  *nnzb = n;
  const size_t MB = (size_t)hdr[0] / hdr[2], nv = (size_t)n * hdr[2] * hdr[3];
  if (row_ptr && col_idx && vals && capacity_blocks >= n) {
    ok = std::fread(row_ptr, sizeof(int), MB + 1, f) == MB + 1 && (!n || std::fread(col_idx, sizeof(int), n, f) == (size_t)n) &&
         (!n || std::fread(vals, elem_size(hdr[4]), nv, f) == nv);
    if (ok && n && hdr[4] == SPMM_F16_SPLIT) ok = vals_lo && std::fread(vals_lo, 2, nv, f) == nv;
    if (ok && n && hdr[4] == SPMM_E4M3) ok = scales && std::fread(scales, sizeof(float), n, f) == (size_t)n;
  }
  std::fclose(f);
  return ok ? SPMM_OK : spmm::host_fail(SPMM_ERR_INVALID_ARG, std::string("truncated BCSR file: ") + path);
}

}  // extern "C"
