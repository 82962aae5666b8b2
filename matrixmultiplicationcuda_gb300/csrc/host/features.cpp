// Structure features of a BCSR product, the input of the learned cost model.
//
// Eighteen numbers, all computable from the shape, the type and the BCSR
// index arrays in one pass over row_ptr and col_idx:
//   0 log2 M             1 log2 K             2 log2 N
//   3 bR == 16           4 bR == 32           5 bR == 64
//   6 log2 block density (stored blocks / block slots, floored at 2^-20)
//   7 log2(1 + mean blocks per block row)
//   8 coefficient of variation of blocks per block row
//   9 log2(1 + max blocks per block row)
//  10 band width: max over stored blocks of |16 * col - bR * row| / K
//  11 fraction of block rows with no blocks
//  12 log2 of the mean run length of consecutive block columns within a row
//  13 log2(block rows x 256-column tiles / 152): work items per SM
//  14 max / mean blocks per block row (load imbalance; 0 for an empty matrix)
//  15 distinct block columns referenced / K * 16 (share of B's rows read)
//  16 bytes per stored A element (2 for fp16, bf16 and split fp16; 1 for e4m3)
//  17 1 for the split hi+lo fp16 product (three MMAs per block), else 0
// The generator's pattern label is not among them: a caller's matrix has
// none. Band width, run length and row-count spread are the structural
// quantities that tell the random, band, block-diagonal and clustered patterns
// apart.
#include <algorithm>
#include <cmath>
#include <vector>
#include "../../../include/bcsr_spmm.h"

extern "C" int spmm_structure_features_host(const int* row_ptr, const int* col_idx, int M, int K, int bR, int N,
                                            spmm_dtype dtype, float* out) {
  if (!row_ptr || !out || M <= 0 || K <= 0 || N <= 0 || bR <= 0 || M % bR || K % 16) return -1;
  if ((int)dtype < 0 || (int)dtype > 3) return -1;
  const int MB = M / bR, KB = K / 16;
  const long long nnzb = row_ptr[MB] - row_ptr[0];
  if (nnzb > 0 && !col_idx) return -1;
  double sum = 0, sq = 0, mx = 0, empty = 0, band = 0, runs = 0;
  std::vector<unsigned char> seen(KB, 0);
  long long distinct = 0;
  for (int r = 0; r < MB; ++r) {
    const int a = row_ptr[r], b = row_ptr[r + 1];
    if (a < row_ptr[0] || b < a || b > row_ptr[MB]) return -1;
    const double n = b - a;
    sum += n;
    sq += n * n;
    mx = std::max(mx, n);
    if (n == 0) empty += 1;
    for (int j = a; j < b; ++j) {
      const int c = col_idx[j];
      if (c < 0 || c >= KB) return -1;
      band = std::max(band, std::fabs(16.0 * c - (double)bR * r));
      if (j == a || c != col_idx[j - 1] + 1) runs += 1;
      if (!seen[c]) {
        seen[c] = 1;
        ++distinct;
      }
    }
  }
  const double mean = sum / MB;
  const double var = std::max(0.0, sq / MB - mean * mean);
  out[0] = (float)std::log2((double)M);
  out[1] = (float)std::log2((double)K);
  out[2] = (float)std::log2((double)N);
  out[3] = bR == 16 ? 1.f : 0.f;
  out[4] = bR == 32 ? 1.f : 0.f;
  out[5] = bR == 64 ? 1.f : 0.f;
  out[6] = (float)std::log2(std::max((double)nnzb / ((double)MB * KB), 1.0 / 1048576.0));
  out[7] = (float)std::log2(1.0 + mean);
  out[8] = (float)(mean > 0 ? std::sqrt(var) / mean : 0.0);
  out[9] = (float)std::log2(1.0 + mx);
  out[10] = (float)(band / K);
  out[11] = (float)(empty / MB);
  out[12] = (float)(runs > 0 ? std::log2((double)nnzb / runs) : 0.0);
  out[13] = (float)std::log2((double)MB * ((N + 255) / 256) / 152.0);
  out[14] = (float)(mean > 0 ? mx / mean : 0.0);
  out[15] = (float)((double)distinct / KB);
  out[16] = dtype == SPMM_E4M3 ? 1.f : 2.f;
  out[17] = dtype == SPMM_F16_SPLIT ? 1.f : 0.f;
  return 0;
}
