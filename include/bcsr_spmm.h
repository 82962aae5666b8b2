/*
 * bcsr_spmm.h -- C ABI of the GB300 (sm_103a) BCSR sparse x dense multiply.
 *
 *   C (M x N, fp32, row-major) = A (M x K, BCSR, bR x 16 blocks) * B (K x N, row-major)
 *
 * Every entry point takes plain pointers and sizes, returns an spmm_status and
 * never aborts. Device pointers are CUDA device (or managed) addresses; a
 * `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 * Launches are asynchronous on that stream unless the comment says otherwise.
 *
 * The BCSR layout is the reference's BCSRMatrix (formats/BCSRMatrix.cuh:9-26,
 * built in formats/BCSRMatrix.cu:22-74): row_ptr ("hdr") has M/bR + 1 ints,
 * col_idx ("idx") has nnzb ints in units of 16 columns of A (= 16 rows of B),
 * and the values hold nnzb blocks of bR x 16 elements, each block row-major and
 * contiguous, blocks in row-major block order.
 */
#ifndef BCSR_SPMM_H
#define BCSR_SPMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum spmm_status {
  SPMM_OK = 0,
  SPMM_ERR_INVALID_ARG = 1,    /* null pointer, negative size, bad block shape   */
  SPMM_ERR_UNSUPPORTED = 2,    /* a shape or dtype the library has no kernel for */
  SPMM_ERR_MISALIGNED = 3,     /* a pointer or leading dimension breaks TMA rules */
  SPMM_ERR_CUDA = 4,           /* a CUDA runtime / driver call failed             */
  SPMM_ERR_TIMEOUT = 5,        /* a bounded device-side wait gave up              */
  SPMM_ERR_BAD_STRUCTURE = 6,  /* row_ptr / col_idx failed validation             */
  SPMM_ERR_SCRATCH_TOO_SMALL = 7
} spmm_status;

/* Storage / arithmetic type of A and B. All accumulate in fp32 and write fp32 C. */
typedef enum spmm_dtype {
  SPMM_F16 = 0,        /* A, B fp16 (the reference's type)                               */
  SPMM_BF16 = 1,       /* A, B bf16                                                      */
  SPMM_E4M3 = 2,       /* A e4m3 + one fp32 scale per block, B e4m3 + one fp32 scale     */
  SPMM_F16_SPLIT = 3   /* A = A_hi + A_lo, B = B_hi + B_lo (fp16 pairs), 3 products      */
} spmm_dtype;

/* Kernel configuration. Zero-initialised = let the library choose. */
typedef struct spmm_config {
  int kernel;    /* 0 = auto, 1 = mma.sync pipeline, 2 = tcgen05 pipeline,
                    3 = tcgen05 pipeline for 64-row blocks with M = 64 UMMAs       */
  int n_tile;    /* output columns per CTA tile: 64, 128 or 256 (0 = auto)           */
  int stages;    /* pipeline depth 2..8 (0 = auto)                                   */
  int ctas_per_sm; /* persistent grid = SMs x this (0 = auto)                          */
  int acc_buffers; /* tcgen05: TMEM accumulators per CTA, 1 or 2 (0 = auto)          */
  int schedule;    /* tcgen05: 0 = static item stride, 1 = atomic work queue,
                      2 = per-matrix plan (a tuner-table mark: spmm_bcsr_plan_create
                      builds the plan, whose runs chain with
                      SPMM_RUN_INPUTS_READY; spmm_bcsr_mm runs it as 1)       */
  int split_k;     /* tcgen05: split each block row's blocks over this many work
                      items whose partial products are added into C (C is
                      zeroed first; the order of the additions varies from run
                      to run). 0 or 1 = no split; at most 16.                   */
} spmm_config;

/* Describes A. All arrays are device pointers. */
typedef struct spmm_bcsr_desc {
  int M, K;              /* rows / columns of A: multiples of bR and 16              */
  int bR, bC;            /* block shape: bR in {16, 32, 64}, bC == 16                */
  const int* row_ptr;    /* M/bR + 1 entries                                         */
  const int* col_idx;    /* nnzb entries (col_idx / vals may be NULL when nnzb == 0)  */
  const void* vals;      /* nnzb * bR * 16 elements of dtype (A_hi for F16_SPLIT)     */
  const void* vals_lo;   /* F16_SPLIT: A_lo, same layout; otherwise NULL             */
  const float* scales;   /* E4M3: nnzb per-block fp32 scales; otherwise NULL         */
  spmm_dtype dtype;
} spmm_bcsr_desc;

/* Describes B (K x N row-major, leading dimension ldb >= N, in elements). */
typedef struct spmm_dense_desc {
  const void* data;      /* K x ldb elements (B_hi for F16_SPLIT)                    */
  const void* data_lo;   /* F16_SPLIT: B_lo; otherwise NULL                          */
  float scale;           /* E4M3: the fp32 scale of B (B = scale * stored); else 1   */
  int ldb;
} spmm_dense_desc;

/* ---- library ------------------------------------------------------------------ */
int spmm_abi_version(void);
/* Text of the last error on the calling host thread ("" if none). */
const char* spmm_last_error(void);

/* ---- general entry point -------------------------------------------------------
 * C[M x N] (ldc >= N, in floats) = A * B. Every C element in the M x N window is
 * written (rows whose block row is empty get zeros), so C need not be cleared.
 * N must be a multiple of 8 and ldb a multiple of 8 (16-byte TMA strides);
 * E4M3 needs multiples of 16. cfg may be NULL.
 * E4M3 with kernel 0 runs the mma.sync pipeline, which takes any fp32 block
 * scale. Kernel 2 runs the tcgen05 block-scaled kernels (kind::mxf8f6f4):
 * every block scale must be a positive normal power of two, as spmm_quantize
 * makes them (another scale raises a flag spmm_device_error_check reports);
 * each 16-wide block is a K = 32 MMA whose second half multiplies zeros by
 * the panel of the next 128 output columns, so a NaN stored in B can reach
 * the C entry 128 columns to its left in rows whose blocks read that B row.
 */
spmm_status spmm_bcsr_mm(const spmm_bcsr_desc* A, const spmm_dense_desc* B, int N,
                         float* C, int ldc, const spmm_config* cfg, void* stream);

/* Checks row_ptr / col_idx on the device (monotone, row_ptr[0] == 0,
 * row_ptr[M/bR] == nnzb, col_idx in [0, K/16), strictly ascending within a
 * row); col_idx is read only after row_ptr passed. Synchronises the stream.
 * The reference never validates (its kernels trust hdr/idx). */
spmm_status spmm_bcsr_validate(const int* row_ptr, const int* col_idx, int M, int K, int bR,
                               long long nnzb, void* stream);

/* ---- reference-shaped launchers ------------------------------------------------
 * Drop-ins for the launch sites of the reference's __global__ kernels
 * (src/cuda_kernels.cuh:39-114): the same argument list (hdr, idx, data, B, C,
 * M, N) with fp16 data and B, plus K (the row count of B, which the
 * reference's kernels never read because they trust idx; every reference call
 * site has it) and the stream of the launch configuration. The grid, block and
 * shared-memory sizes are chosen here. */

/* 16x16 blocks: src/cuda_kernels.cu:301-328 (launch nvbench_main.cu:339-346).   */
spmm_status sparseMatrixMulTensor_launch(const int* hdr, const int* idx, const void* data,
                                         const void* B, float* C, unsigned M, unsigned N,
                                         unsigned K, void* stream);
/* 32x16 blocks: src/cuda_kernels.cu:699-762 (launch nvbench_main.cu:648-655).   */
spmm_status sparseMatrixMulTensor32x16_launch(const int* hdr, const int* idx, const void* data,
                                              const void* B, float* C, unsigned M, unsigned N,
                                              unsigned K, void* stream);
/* 64x16 blocks: src/cuda_kernels.cu:618-695 (launch nvbench_main.cu:548-555).   */
spmm_status sparseMatrixMulTensor64x16_launch(const int* hdr, const int* idx, const void* data,
                                              const void* B, float* C, unsigned M, unsigned N,
                                              unsigned K, void* stream);
/* The reference's variant kernels compute the same product with other warp
 * splits or staging. Each has a launcher of its own name, with the argument
 * list above, that runs this library's pipeline for its block shape. */
/* sparseMatrixMulTensor_v2, src/cuda_kernels.cu:370-417 (16x16) */
spmm_status sparseMatrixMulTensor_v2_launch(const int* hdr, const int* idx, const void* data,
                                            const void* B, float* C, unsigned M, unsigned N,
                                            unsigned K, void* stream);
/* sparseMatrixMulTensor_v3, src/cuda_kernels.cu:423-489 (16x16) */
spmm_status sparseMatrixMulTensor_v3_launch(const int* hdr, const int* idx, const void* data,
                                            const void* B, float* C, unsigned M, unsigned N,
                                            unsigned K, void* stream);
/* sparseMatrixMulTensor_v1_improved, src/cuda_kernels.cu:495-547 (16x16) */
spmm_status sparseMatrixMulTensor_v1_improved_launch(const int* hdr, const int* idx, const void* data,
                                                     const void* B, float* C, unsigned M, unsigned N,
                                                     unsigned K, void* stream);
/* sparseMatrixMulTensor_option2_ldmatrix_sm80, src/cuda_kernels.cu:552-613 (16x16) */
spmm_status sparseMatrixMulTensor_option2_ldmatrix_sm80_launch(const int* hdr, const int* idx, const void* data,
                                                               const void* B, float* C, unsigned M, unsigned N,
                                                               unsigned K, void* stream);
/* sparseMatrixMulTensor1, src/cuda_kernels.cu:330-355 (16x16, square n x n
 * matrices: M = N = K = n, the reference's parameter list plus a stream) */
spmm_status sparseMatrixMulTensor1_launch(const int* hdr, const int* idx, const void* data, const void* B,
                                          float* C, unsigned n, void* stream);
/* sparseMatrixMulTensor32x16_v2, src/cuda_kernels.cu:1001-1050 (32x16) */
spmm_status sparseMatrixMulTensor32x16_v2_launch(const int* hdr, const int* idx, const void* data,
                                                 const void* B, float* C, unsigned M, unsigned N,
                                                 unsigned K, void* stream);
/* sparseMatrixMulTensor32x16_shared, src/cuda_kernels.cu:768-845 (32x16) */
spmm_status sparseMatrixMulTensor32x16_shared_launch(const int* hdr, const int* idx, const void* data,
                                                     const void* B, float* C, unsigned M, unsigned N,
                                                     unsigned K, void* stream);
/* sparseMatrixMulTensor32x16_shared_vectorized, src/cuda_kernels.cu:853-934 (32x16) */
spmm_status sparseMatrixMulTensor32x16_shared_vectorized_launch(const int* hdr, const int* idx,
                                                                const void* data, const void* B, float* C,
                                                                unsigned M, unsigned N, unsigned K,
                                                                void* stream);
/* sparseMatrixMulTensor32x16_v2_shared_vectorized, src/cuda_kernels.cu:1056-1166 (32x16) */
spmm_status sparseMatrixMulTensor32x16_v2_shared_vectorized_launch(const int* hdr, const int* idx,
                                                                   const void* data, const void* B,
                                                                   float* C, unsigned M, unsigned N,
                                                                   unsigned K, void* stream);
/* sparseMatrixMulTensor64x16_v2, src/cuda_kernels.cu:939-996 (64x16) */
spmm_status sparseMatrixMulTensor64x16_v2_launch(const int* hdr, const int* idx, const void* data,
                                                 const void* B, float* C, unsigned M, unsigned N,
                                                 unsigned K, void* stream);
/* Adaptive / Adaptive32x16 / Adaptive64x16 (src/cuda_kernels.cu:1171-1363):
 * colBlocksPerRow is accepted and ignored (the persistent schedule balances the
 * columns). */
spmm_status sparseMatrixMulTensorAdaptive_launch(const int* hdr, const int* idx, const void* data,
                                                 const void* B, float* C, unsigned M, unsigned N,
                                                 unsigned colBlocksPerRow, unsigned K, void* stream);
spmm_status sparseMatrixMulTensorAdaptive32x16_launch(const int* hdr, const int* idx,
                                                      const void* data, const void* B, float* C,
                                                      unsigned M, unsigned N,
                                                      unsigned colBlocksPerRow, unsigned K,
                                                      void* stream);
spmm_status sparseMatrixMulTensorAdaptive64x16_launch(const int* hdr, const int* idx,
                                                      const void* data, const void* B, float* C,
                                                      unsigned M, unsigned N,
                                                      unsigned colBlocksPerRow, unsigned K,
                                                      void* stream);

/* ---- dense -> BCSR on the GPU (BCSRMatrix ctor, formats/BCSRMatrix.cu:22-74) ---
 * Bit-exact to the reference: a block is kept when any of its fp16 elements
 * compares != 0 as a float (so -0 is zero and NaN is not), blocks in row-major
 * block order, explicit zeros inside kept blocks are stored.
 * Step 1 writes row_ptr (M/bR + 1 ints, device) and returns nnzb in *nnzb_out
 * (synchronises the stream). Step 2 fills col_idx (nnzb ints) and vals
 * (nnzb * bR * bC halves). A is M x K fp16 row-major on the device, lda >= K.
 * Block sizes follow the ctor's checks (:24-34): multiples of 16, >= 16; this
 * library's kernels then need bC == 16. M and K are truncated to whole blocks
 * like the ctor (:37-38). */
spmm_status spmm_dense_to_bcsr_count(const void* A, int M, int K, int lda, int bR, int bC,
                                     int* row_ptr, long long* nnzb_out, void* stream);
spmm_status spmm_dense_to_bcsr_fill(const void* A, int M, int K, int lda, int bR, int bC,
                                    const int* row_ptr, int* col_idx, void* vals, void* stream);

/* ---- generators on the GPU ------------------------------------------------------
 * The host generators' counter-based streams (bcsr_spmm_host.h), evaluated on
 * the device, for inputs too large to generate on the host quickly.
 *   gen_structure: as spmm_gen_structure into device row_ptr (M/bR + 1) and
 *     col_idx (capacity entries; skipped when too small or NULL); *nnzb_out is
 *     always set (synchronises the stream). Random, band and block-diagonal
 *     structures are bit-identical to the host's; log-normal row counts go
 *     through device log / exp, so one may differ by one from the host's.
 *   gen_values / gen_dense: as spmm_gen_values / spmm_gen_dense (uniform
 *     values bit-identical, normal ones the same transform).
 *   generate_matrix: a dense fp16 matrix in one of the reference generator's
 *     patterns (matrix_generator.cpp:28-140) with the counter-based stream
 *     instead of mt19937: the same shapes and value distribution, not the
 *     reference's bits (spmm_generate_matrix is the bit-identical host one). */
spmm_status spmm_gpu_gen_structure(int M, int K, int bR, int pattern, double density, double param,
                                   unsigned long long seed, int* row_ptr, int* col_idx,
                                   long long capacity, long long* nnzb_out, void* stream);
spmm_status spmm_gpu_gen_values(long long nnzb, int bR, int bC, int dist, unsigned long long seed,
                                float* out, void* stream);
spmm_status spmm_gpu_gen_dense(long long count, int dist, unsigned long long seed, float* out,
                               void* stream);
spmm_status spmm_gpu_generate_matrix(int rows, int cols, double sparsity, const char* pattern,
                                     int blocksize, unsigned long long seed, void* out_half,
                                     void* stream);

/* ---- precision conversion (device, asynchronous) ------------------------------
 * From fp32 block values (the exact values before storage rounding):
 *   to fp16 / bf16 (round to nearest even),
 *   to e4m3 with one scale per block (scale = the smallest power of two >= max|block| / 448,
 *     1 for all-zero blocks; a power of two is what the tcgen05 e4m3 kernels need),
 *   to an fp16 hi/lo pair (hi = fp16(x), lo = fp16(x - hi)).
 * `count` elements, `block_elems` elements per scale block (E4M3 only). */
spmm_status spmm_quantize(const float* src, size_t count, spmm_dtype dtype, int block_elems,
                          void* dst, void* dst_lo, float* scales, void* stream);

/* ---- batched: many independent SpMMs in one persistent launch -----------------
 * problems[i] describes one product; all must share dtype (F16 or BF16).
 * The launch walks one work queue of (problem, block row, column tile) items,
 * heaviest first. `plan` is an opaque host handle built once per batch
 * (it owns a device copy of the problem table and the ordered queue).
 * A 16- or 32-row problem (M a multiple of 64) whose block rows share most of
 * their columns (the union of each 64 rows' columns holds at most 60 % of the
 * blocks, as in band and block-diagonal structures) runs stacked, as a
 * per-matrix plan runs it: 64-row blocks over that union, zeros where a row
 * has no block. The launch assembles each stacked block in shared memory
 * from its member blocks, read from the problem's own values (rows with no
 * block read zeros), so a run takes the current values and needs no copy.
 * Such a problem's column indices must stay those the plan was built from;
 * its values may change between runs. */
typedef struct spmm_problem {
  spmm_bcsr_desc A;
  spmm_dense_desc B;
  int N;
  float* C;
  int ldc;
} spmm_problem;
typedef struct spmm_batch_plan spmm_batch_plan;
/* cfg (NULL: defaults): n_tile 0 (128 columns for N <= 128, else 256), 128 or
 * 256; stages 0, 2, 4 or 8 (the ring in groups: two groups of four blocks by
 * default, four groups of two when some problem runs stacked, eight of one);
 * ctas_per_sm 0 (as many as fit, at most 2) or fewer. */
spmm_status spmm_batch_plan_create(const spmm_problem* problems, int count,
                                   const spmm_config* cfg, spmm_batch_plan** plan_out);
spmm_status spmm_batch_run(const spmm_batch_plan* plan, void* stream);
/* Items of the launch, and problems run stacked (no counterpart in the reference). */
spmm_status spmm_batch_plan_info(const spmm_batch_plan* plan, int* items, int* stacked_problems);
spmm_status spmm_batch_plan_destroy(spmm_batch_plan* plan);

/* ---- hybrid BCSR + CSR (HCSRMatrix, formats/HCSRMatrix.cpp:10-36) -------------
 * C = A_blocks B + A_rest B in ONE launch: the tcgen05 pipeline multiplies the
 * BCSR part (any block height; the reference uses 16 x 16), and its epilogue
 * warps add the CSR part's entries to each tile after storing it. The reference
 * runs three kernels (CSR into a second buffer, BCSR into C, then an
 * element-wise add; main.cu:567-590). fp16 only, no split-K. Both parts
 * describe the same M x K matrix; A_rest->row_ptr has M + 1 entries, col_idx
 * holds column indices (not the reference's i % rows). */
typedef struct spmm_csr_desc {
  int M, K;
  const int* row_ptr;
  const int* col_idx;
  const void* vals;      /* fp16 */
} spmm_csr_desc;
spmm_status spmm_hcsr_mm(const spmm_bcsr_desc* A_blocks, const spmm_csr_desc* A_rest,
                         const spmm_dense_desc* B, int N, float* C, int ldc,
                         const spmm_config* cfg, void* stream);
/* The hybrid product with a plan: the CSR part is packed once into gather
 * blocks (16 entries of one 16-row block row each, as a 16 x 16 block whose
 * column c holds entry c, plus the entries' 16 B-row indices). The tcgen05
 * pipeline then runs stored and gather blocks alike on the tensor cores, and
 * fetches a gather block's B rows with TMA tile::gather4. 16 x 16 fp16 blocks.
 * _create reads both parts on the device and synchronises `stream` once (for
 * the sizes). The plan owns its arrays: the parts may be freed after _create.
 * _run only launches (one kernel; no allocation or synchronisation); any N,
 * ldb, ldc, configuration and split-K of kernel 2. */
typedef struct spmm_hcsr_plan spmm_hcsr_plan;
spmm_status spmm_hcsr_plan_create(const spmm_bcsr_desc* A_blocks, const spmm_csr_desc* A_rest,
                                  void* stream, spmm_hcsr_plan** plan_out);
spmm_status spmm_hcsr_plan_info(const spmm_hcsr_plan* plan, long long* blocks,
                                long long* gather_blocks);
spmm_status spmm_hcsr_plan_run(const spmm_hcsr_plan* plan, const spmm_dense_desc* B, int N,
                               float* C, int ldc, const spmm_config* cfg, void* stream);
spmm_status spmm_hcsr_plan_destroy(spmm_hcsr_plan* plan);
/* CSR x dense (fp16 A and B, fp32 C), the comparator beside the BCSR path. It
 * replaces the reference's scalar CSR kernel (src/cuda_kernels.cu:271-299, one
 * thread per output element) with one warp per row and 256 columns. N % 8 == 0,
 * B and C 16-byte aligned. Asynchronous. */
spmm_status spmm_csr_mm(const spmm_csr_desc* A, const spmm_dense_desc* B, int N, float* C, int ldc,
                        void* stream);

/* Dense x dense (fp16 or bf16 A and B, fp32 C) on the tcgen05 tensor cores: the
 * native dense comparator. It replaces the reference's denseMatrixMulTensor
 * (src/cuda_kernels.cu:246-270, one WMMA warp per 16 x 16 tile) and its scalar
 * dense kernels (src/cuda_kernels.cu:86-244). A is M x K row-major (lda >= K, a
 * multiple of 8), B K x N row-major (ldb >= N, a multiple of 8), C M x N fp32
 * (ldc >= N, a multiple of 4); N % 8 == 0; 16-byte aligned bases. Asynchronous. */
spmm_status spmm_dense_mm(const void* A, int lda, const spmm_dense_desc* B, int M, int K, int N,
                          spmm_dtype dtype, float* C, int ldc, void* stream);

/* ---- tuning ----------------------------------------------------------------------
 * No counterpart in the reference (its harness sweeps kernels by hand).
 * The configuration space: a fixed table of spmm_tune_config_count() entries
 * (41: five mma.sync column tiles and depths; tcgen05 column tiles, depths,
 * accumulator counts, static or work-queue schedules and split-K; the 64-row
 * tcgen05 pipeline's column tiles and schedules). Not every entry has a kernel
 * for every block height and type. */
int spmm_tune_config_count(void);
spmm_status spmm_tune_config(int i, spmm_config* out);
/* The configuration spmm_bcsr_mm runs when given none (the library's fixed
 * heuristic), as a table entry. */
spmm_status spmm_default_config(int bR, spmm_dtype dtype, int N, spmm_config* out);
/* SPMM_OK if `cfg` has a kernel for (bR, dtype, N), else SPMM_ERR_UNSUPPORTED. */
spmm_status spmm_config_supported(int bR, spmm_dtype dtype, int N, const spmm_config* cfg);
/* Exhaustive sweep: times every table entry on this product. Per entry:
 * `warmup` untimed runs, then `reps` runs each preceded (when flush != NULL)
 * by a write of flush_bytes to `flush` (evicting L2) and timed alone with CUDA
 * events; ms_out[i] = the mean, +inf where the entry has no kernel. A plan
 * entry (schedule 2) builds the plan once and times its runs.
 * Overwrites C; synchronises the stream. */
spmm_status spmm_tune_sweep(const spmm_bcsr_desc* A, const spmm_dense_desc* B, int N, float* C, int ldc,
                            int warmup, int reps, void* flush, size_t flush_bytes, float* ms_out,
                            void* stream);

/* Back-to-back sweep: times every table entry as `launches` consecutive
 * products over the `ncopies` copies of one problem (copy k % ncopies for
 * launch k; copies large enough together to exceed L2 make every launch read
 * its inputs from HBM), captured in one CUDA graph and replayed after `warmup`
 * eager runs and one untimed replay (launches issued one by one if capture
 * fails). Plan entries (schedule 2) build one plan from copies[0] and chain
 * their runs with SPMM_RUN_INPUTS_READY. ms_out[i] = the mean time per launch,
 * +inf where the entry has no kernel. This is the regime of a caller that
 * runs product after product on one stream. Overwrites every copy's C;
 * synchronises. */
spmm_status spmm_tune_sweep_b2b(const spmm_problem* copies, int ncopies, int launches, int warmup,
                                float* ms_out, void* stream);

/* Structure features (18 floats) of the product A (M x K, bR x 16 blocks,
 * element type dtype) x B (K x N), the cost model's input. The _host variant
 * reads host arrays and returns 0 (or -1 on a bad structure); the other copies
 * row_ptr and col_idx from the device and synchronises the stream. */
#define SPMM_FEATURES 18
int spmm_structure_features_host(const int* row_ptr, const int* col_idx, int M, int K, int bR, int N,
                                 spmm_dtype dtype, float* out);
spmm_status spmm_structure_features(const spmm_bcsr_desc* A, int N, float* out, void* stream);

/* ---- learned cost model -------------------------------------------------------
 * No counterpart in the reference. A fp32 MLP: features -> normalisation ->
 * `layers` hidden layers of `hidden` units with GELU -> `out` outputs,
 * ln(microseconds) per tuner configuration. Parameters are one flat array
 * (mu[in], sigma[in], then per layer W[fan_out x fan_in] row-major and
 * b[fan_out]). Forward, backward (masked mean squared error) and Adam run in
 * the library's own kernels on device arrays, asynchronously on `stream`. */
typedef struct spmm_mlp_shape {
  int in, hidden, layers, out;   /* in, hidden <= 128; out <= 1024; layers <= 16;
                                    a model for spmm_cost_model_create has in ==
                                    SPMM_FEATURES and out == spmm_tune_config_count() */
} spmm_mlp_shape;
long long spmm_mlp_param_count(const spmm_mlp_shape* shape);
long long spmm_mlp_workspace_floats(const spmm_mlp_shape* shape, int batch);
/* Y[batch x out] from X[batch x in]. */
spmm_status spmm_mlp_forward(const spmm_mlp_shape* shape, const float* params, const float* X, int batch,
                             float* Y, float* work, void* stream);
/* loss = sum(mask * (Y - T)^2) / sum(mask) (one float, may be NULL) and
 * grad = d loss / d params (zero for mu and sigma). */
spmm_status spmm_mlp_backward(const spmm_mlp_shape* shape, const float* params, const float* X,
                              const float* T, const float* mask, int batch, float* grad, float* loss,
                              float* work, void* stream);
/* One AdamW step (decoupled weight decay) on params[offset, n). step >= 1. */
spmm_status spmm_mlp_adam(float* params, const float* grad, float* m, float* v, long long n,
                          long long offset, float lr, float beta1, float beta2, float eps,
                          float weight_decay, int step, void* stream);
/* A trained model on the current device (parameters copied from the host;
 * `out` must equal spmm_tune_config_count()). select computes the features
 * of A, runs the network and returns the supported configuration with the
 * smallest predicted time (and, if `predicted_ms` is not NULL, every
 * entry's prediction in ms, +inf where unsupported). Synchronises the stream. */
typedef struct spmm_cost_model spmm_cost_model;
spmm_status spmm_cost_model_create(const spmm_mlp_shape* shape, const float* host_params,
                                   spmm_cost_model** out);
/* The same from a file: "SPMMCM01", int32 in, hidden, layers, out, then the
 * fp32 parameters (little-endian). */
spmm_status spmm_cost_model_load(const char* path, spmm_cost_model** out);
spmm_status spmm_cost_model_destroy(spmm_cost_model* model);
spmm_status spmm_cost_model_select(const spmm_cost_model* model, const spmm_bcsr_desc* A, int N,
                                   spmm_config* out, float* predicted_ms, void* stream);

/* ---- per-matrix plan (tcgen05 pipeline) ----------------------------------------
 * A launch is bound by its longest CTA, and one block row (and column tile) is
 * one CTA's item. _create reads row_ptr once (it synchronises `stream`) and
 * builds an item list ordered heaviest first. A row longer than 3x the
 * average load per CTA slot is cut into parts of about that load, run by
 * different CTAs: part 0 zeroes the row's C tile while its MMAs run, and
 * every part adds its tile into C with red.add (so C of those rows is summed
 * in an order that varies from run to run within fp32 rounding). The CTAs
 * take the items from the plan's own work queue, each claiming its next item
 * shortly before it has copied the current one, so that CTAs that run faster
 * take more of the lighter items at the end of the list. _run is one launch;
 * A must have the plan's M, K, block shape, dtype and row_ptr (column indices
 * and values may differ), and N must be the plan's. One plan runs one launch
 * at a time (its queue and counters are its own; use one plan per stream for
 * concurrent launches). cfg: kernel 0 or 2, no split-K, schedule 0 or 1
 * (either way the plan's own queue; _info reports schedule 1).
 * 16- and 32-row blocks (fp16 / bf16, M a multiple of 64, N > 256): when the 4 (or 2)
 *   block rows that make up 64 rows of C share most of their block columns
 *   (the union holds at most 60 % of their blocks, as in band and
 *   block-diagonal structures), the plan stacks them into 64-row blocks with
 *   zeros where a row has no block, and a run is one launch of the 64-row
 *   pipeline that assembles each stacked block in shared memory from A's own
 *   blocks: one UMMA and one B panel for up to 4 blocks. A stacked plan is
 *   built from col_idx as well, so A's column indices must stay the plan's;
 *   its values may change, and it takes the early start of
 *   SPMM_RUN_INPUTS_READY like any plan.
 * spmm_bcsr_plan_info: item count, split rows (row and column-tile pairs),
 * and the configuration the plan runs (for a stacked plan, the 64-row one).
 * spmm_bcsr_plan_stacking: block rows per stacked row (1: not stacked) and
 * the stacked blocks. */
typedef struct spmm_bcsr_plan spmm_bcsr_plan;
spmm_status spmm_bcsr_plan_create(const spmm_bcsr_desc* A, int N, const spmm_config* cfg, void* stream,
                                  spmm_bcsr_plan** plan_out);
spmm_status spmm_bcsr_plan_info(const spmm_bcsr_plan* plan, int* items, int* split_rows, spmm_config* cfg);
spmm_status spmm_bcsr_plan_run(const spmm_bcsr_plan* plan, const spmm_bcsr_desc* A, const spmm_dense_desc* B,
                               int N, float* C, int ldc, void* stream);
/* _run with flags (_run is _run_ex with flags 0).
 * SPMM_RUN_INPUTS_READY: the caller promises that no kernel launched on
 *   `stream` since the stream was last synchronised with the host writes A's
 *   arrays or B (constant operands, or a sequence of independent products
 *   whose inputs were all prepared first). The launch may then copy and
 *   multiply its first items while the kernel before it on the stream is
 *   still running (programmatic dependent launch); it still waits for that
 *   kernel before it claims work from the plan's queue and before it writes
 *   C. Without the promise the flag may read stale A or B. */
#define SPMM_RUN_INPUTS_READY 1u
spmm_status spmm_bcsr_plan_run_ex(const spmm_bcsr_plan* plan, const spmm_bcsr_desc* A, const spmm_dense_desc* B,
                                  int N, float* C, int ldc, unsigned flags, void* stream);
spmm_status spmm_bcsr_plan_stacking(const spmm_bcsr_plan* plan, int* rows_per_stack, long long* stacked_blocks);
spmm_status spmm_bcsr_plan_destroy(spmm_bcsr_plan* plan);

/* ---- allocation-free variant ---------------------------------------------------
 * No counterpart in the reference. For callers that cannot call cudaMalloc (a
 * host application or allocator that owns all device memory, a memory budget
 * that forbids the CUDA allocator, code that must not allocate while a stream
 * is being captured): the same product as spmm_bcsr_mm on the tcgen05 pipeline
 * with its work queue, but its scratch -- the device error word and the
 * queue's two counters, 12 bytes -- lives in a fixed 256-byte __device__ array
 * compiled into the library (held on every GPU that loads the library until
 * the process exits), and the call allocates nothing. The caller still passes
 * A, B and C.
 *  - fp16, bf16 and split fp16 only (E4M3 runs on a path with allocated scratch).
 *  - Fewer than 2^30 work items (block rows x column tiles of the tile that
 *    runs x split-K slices): the queue counters are 32-bit. Larger problems
 *    return SPMM_ERR_SCRATCH_TOO_SMALL.
 *  - K == 0 zeroes the C window (cudaMemset2DAsync, which allocates nothing).
 *  - The first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress) and keeps it for the life of the process; make that
 *    first call before any stream capture, and do not use this variant on a
 *    device after cudaDeviceReset (the array may move).
 *  - Every call shares the array (one copy per device) and clears it on its
 *    stream first; calls whose launches overlap on the same GPU (for example on
 *    two streams) race on it, so serialise them.
 * spmm_noalloc_error_check synchronises the stream and reports a timed-out
 * pipeline wait of the last allocation-free call (SPMM_ERR_TIMEOUT). */
spmm_status spmm_bcsr_mm_noalloc(const spmm_bcsr_desc* A, const spmm_dense_desc* B, int N,
                                 float* C, int ldc, const spmm_config* cfg, void* stream);
spmm_status spmm_noalloc_error_check(void* stream);

/* ---- diagnostics ---------------------------------------------------------------
 * Runs one block of the pipeline's bounded mbarrier wait on a barrier that no
 * one arrives on, with the given limit in nanoseconds; returns SPMM_ERR_TIMEOUT
 * when the wait gave up and the kernel exited cleanly (synchronises). */
spmm_status spmm_debug_wait_timeout(unsigned long long timeout_ns, void* stream);
/* Synchronises the stream, then reads and clears the device error word that the
 * pipelines set when a bounded wait gives up; SPMM_ERR_TIMEOUT if it was set.
 * SPMM_ERR_INVALID_ARG when the only flag is the tcgen05 e4m3 kernels' scale
 * check (a block scale that is not a positive normal power of two; that
 * product used the scale's exponent alone). */
spmm_status spmm_device_error_check(void* stream);
/* Number of SMs of the current device (for grid sizing in callers). */
int spmm_device_sm_count(void);

#ifdef __cplusplus
}
#endif
#endif /* BCSR_SPMM_H */
