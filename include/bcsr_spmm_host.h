/* Host-side C API of libbcsr_spmm: seeded generators, the .mat text format and
 * host construction of the BCSR / CSR layouts. No GPU needed; thread-safe.
 * Errors are reported through spmm_last_error (bcsr_spmm.h). */
#ifndef BCSR_SPMM_HOST_H
#define BCSR_SPMM_HOST_H
#include <stddef.h>
#include "bcsr_spmm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* mg::generate_matrix<float>(rows, cols, sparsity, pattern, blocksize, seed)
 * (matrix_generator.cpp:28-140): the same patterns, std::mt19937 stream and
 * draw order, so the matrix is bit-identical to the reference's. Writes a
 * row-major fp32 rows x cols buffer; -1 on an unknown pattern. */
int spmm_generate_matrix(int rows, int cols, double sparsity, const char* pattern, int blocksize,
                         unsigned seed, float* out);

/* Block structure of an M x K matrix with bR x 16 blocks (no reference
 * counterpart: the reference's patterns are element patterns).
 *   pattern 0 random:    each block kept with probability `density`;
 *   pattern 1 band:      blocks within `param` block columns of the diagonal,
 *                        each kept with probability min(1, density*KB / band length);
 *   pattern 2 blockdiag: dense diagonal tiles of `param` x `param` elements;
 *   pattern 3 lognormal: per-row counts ~ LogNormal(mean density*KB, CV `param`),
 *                        columns uniform without replacement.
 * row_ptr holds M/bR + 1 entries, col_idx room for (M/bR) * (K/16). Returns
 * nnzb, or -1 on bad arguments. */
long long spmm_gen_structure(int M, int K, int bR, int pattern, double density, double param,
                             unsigned long long seed, int* row_ptr, int* col_idx);

/* fp32 values of nnzb blocks of bR x bC: dist 0 uniform[-1, 1]; dist 1
 * N(0,1) x 10^u per block, u ~ uniform[-3, 3]; dist 2 N(0,1). Counter-based,
 * so the output does not depend on thread count. */
void spmm_gen_values(long long nnzb, int bR, int bC, int dist, unsigned long long seed, float* out);
/* `count` dense fp32 values: dist 0 uniform[-1, 1], dist 2 N(0,1). */
void spmm_gen_dense(long long count, int dist, unsigned long long seed, float* out);

/* The .mat text format (Matrix.cu:14-32; written by matrix_generator.py:110-122):
 * "rows cols" then rows*cols values, row-major. load rounds to fp16 (bits in
 * out_half) and counts nonZeros as the reference does. */
spmm_status spmm_mat_read_header(const char* path, int* rows, int* cols);
spmm_status spmm_mat_load(const char* path, void* out_half, size_t capacity, int* rows, int* cols,
                          int* nonZeros);
spmm_status spmm_mat_save(const char* path, const float* vals, int rows, int cols);

/* BCSRMatrix(matrix, bR, bC) on the host (formats/BCSRMatrix.cu:22-74):
 * returns nnzb and fills hdr / idx / vals (fp16 bits) when they are non-NULL;
 * -1 on a block shape the reference rejects. */
long long spmm_host_dense_to_bcsr(const void* A_half, int rows, int cols, int bR, int bC, int* hdr,
                                  int* idx, void* vals);
/* CSRMatrix(matrix) (formats/CSRMatrix.cu:10-43) with the column index of
 * element i stored as i % cols (the reference stores i). Returns nnz. */
long long spmm_host_dense_to_csr(const void* A_half, int rows, int cols, int* hdr, int* idx,
                                 void* vals);

/* The per-matrix plan's item list (spmm_bcsr_plan_create, bcsr_spmm.h) on
 * the host, for row_ptr (MB + 1 entries), `ntiles` column tiles and `slots`
 * CTA slots (SMs x CTAs per SM): rows longer than 3x the average load per
 * slot cut into parts, items ordered heaviest first (the parts of a row
 * together, part 0 first). items: 4 ints per item {block row, column tile,
 * first block, end block}; pair: -1, or 128 * group + part; parts: parts per
 * group. Pass NULL arrays to get *n_items and *n_groups first. */
spmm_status spmm_bcsr_plan_items(const int* row_ptr, int MB, int ntiles, long long slots, int* n_items,
                                 int* n_groups, int* items, int* pair, int* parts);

/* The structure a per-matrix plan stacks 16- or 32-row blocks into (no GPU):
 * each group of `rows_per_stack` block rows becomes one row whose columns are
 * the sorted union of the group's block columns; s_map holds, per stacked
 * block and member row, the source block index or -1 (the block is zeros
 * there). s_row_ptr: MB / rows_per_stack + 1 entries; s_col_idx:
 * *stacked_blocks; s_map: *stacked_blocks * rows_per_stack. Pass NULL arrays
 * to get *stacked_blocks first. SPMM_ERR_INVALID_ARG when a block row repeats
 * a column. */
spmm_status spmm_bcsr_stack_structure(const int* row_ptr, const int* col_idx, int MB, int rows_per_stack,
                                      long long* stacked_blocks, int* s_row_ptr, int* s_col_idx, int* s_map);

/* Matrix Market files (.mtx): what the reference's generator writes through
 * scipy's mmwrite (matrix_generator.py:100-108). Coordinate (real, integer or
 * pattern; general, symmetric or skew-symmetric) and array (real, general)
 * files; repeated entries are summed.
 *   read_header: rows, cols, stored entries.
 *   load:        into a dense row-major fp16 matrix (as Matrix(".mat")).
 *   load_bcsr:   straight into BCSR (bR x bC blocks, fp16, a block kept when
 *                a value in it rounds to a nonzero fp16) without a dense copy:
 *                call with col_idx / vals NULL (or capacity_blocks < nnzb)
 *                for rows, cols, row_ptr (rows/bR + 1 ints) and nnzb, then
 *                with room for nnzb blocks.
 *   save:        a dense fp32 matrix as coordinate real general. */
spmm_status spmm_mtx_read_header(const char* path, int* rows, int* cols, long long* entries);
spmm_status spmm_mtx_load(const char* path, void* out_half, size_t capacity, int* rows, int* cols,
                          int* nonZeros);
spmm_status spmm_mtx_load_bcsr(const char* path, int bR, int bC, int* rows, int* cols, int* row_ptr,
                               long long* nnzb, int* col_idx, void* vals, long long capacity_blocks);
spmm_status spmm_mtx_save(const char* path, const float* vals, int rows, int cols);

/* Binary BCSR file: "SPMMBCS1", int32 M, K, bR, bC, dtype, 0, int64 nnzb,
 * then row_ptr, col_idx, vals (nnzb*bR*bC elements of the dtype), vals_lo
 * (F16_SPLIT) and scales (E4M3), little-endian, as they lie in memory. load:
 * call with NULL arrays (or capacity_blocks < nnzb) for the header, then with
 * room for nnzb blocks. */
spmm_status spmm_bcsr_save(const char* path, int M, int K, int bR, int bC, int dtype, long long nnzb,
                           const int* row_ptr, const int* col_idx, const void* vals, const void* vals_lo,
                           const float* scales);
spmm_status spmm_bcsr_load(const char* path, int* M, int* K, int* bR, int* bC, int* dtype,
                           long long* nnzb, int* row_ptr, int* col_idx, void* vals, void* vals_lo,
                           float* scales, long long capacity_blocks);

/* HCSRMatrix(matrix, threshold) on the host (formats/HCSRMatrix.cpp:10-36):
 * 16x16 blocks with density >= threshold form a BCSR part (bhdr[rows/16 + 1],
 * bidx[nnzb], bvals[nnzb * 256] fp16 bits), all other elements a CSR part
 * (chdr[rows + 1], cidx[nnz], cvals[nnz]). Call once with NULL arrays for the
 * sizes. rows and cols must be multiples of 16. Returns 0, or -1. */
int spmm_host_dense_to_hcsr(const void* A_half, int rows, int cols, float threshold, long long* nnzb,
                            long long* nnz, int* bhdr, int* bidx, void* bvals, int* chdr, int* cidx,
                            void* cvals);

#ifdef __cplusplus
}
#endif
#endif
