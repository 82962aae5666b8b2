// C ABI of libbcsr_spmm: argument checks, error reporting and dispatch.
#include <cudaTypedefs.h>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include "internal.h"

namespace spmm {

namespace {
thread_local std::string g_last_error;
std::mutex g_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
constexpr int kMaxDevices = 64;
unsigned* g_err_word[kMaxDevices] = {nullptr};
int g_sms[kMaxDevices] = {0};

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return -1;
  return d;
}
}  // namespace

spmm_status fail(spmm_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

spmm_status host_fail(spmm_status st, const std::string& msg) { return fail(st, msg); }

void clear_error() { g_last_error.clear(); }

spmm_status cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return SPMM_ERR_CUDA;
}

int sm_count() {
  int d = current_device();
  if (d < 0 || d >= kMaxDevices) return 1;
  if (g_sms[d] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
    g_sms[d] = n > 0 ? n : 1;
  }
  return g_sms[d];
}

int smem_per_sm() {
  static int cache[kMaxDevices] = {0};
  int d = current_device();
  if (d < 0 || d >= kMaxDevices) return 0;
  if (cache[d] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerMultiprocessor, d);
    cache[d] = n;
  }
  return cache[d];
}

namespace {
// Per-device caches of kernel attributes (keyed by kernel address).
struct FnKey {
  const void* fn;
  int dev, a, b;
  bool operator==(const FnKey& o) const { return fn == o.fn && dev == o.dev && a == o.a && b == o.b; }
};
struct FnVal {
  FnKey k;
  int v;
};
std::vector<FnVal> g_fn_cache;
}  // namespace

cudaError_t ensure_smem_attr(const void* fn, int bytes) {
  const FnKey k{fn, current_device(), bytes, -1};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    for (const FnVal& e : g_fn_cache)
      if (e.k == k) return cudaSuccess;
  }
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_fn_cache.push_back({k, 1});
  }
  return e;
}

int max_blocks_per_sm(const void* fn, int threads, size_t smem) {
  const FnKey k{fn, current_device(), threads, (int)smem};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    for (const FnVal& e : g_fn_cache)
      if (e.k == k) return e.v;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess) n = 1;
  std::lock_guard<std::mutex> lk(g_mu);
  g_fn_cache.push_back({k, n});
  return n;
}

bool pdl_enabled() {
  static const bool on = std::getenv("SPMM_NO_PDL") == nullptr;
  return on;
}

unsigned* device_error_word() {
  int d = current_device();
  if (d < 0 || d >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_err_word[d]) {
    void* p = nullptr;
    if (cudaMalloc(&p, 256) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, 256) != cudaSuccess) return nullptr;
    g_err_word[d] = static_cast<unsigned*>(p);
  }
  return g_err_word[d];
}

namespace {
constexpr int kQueueSlots = 256;
unsigned* g_queue_pool[kMaxDevices] = {nullptr};
unsigned g_queue_next[kMaxDevices] = {0};
}  // namespace

unsigned* work_queue_slot() {
  int d = current_device();
  if (d < 0 || d >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_queue_pool[d]) {
    void* p = nullptr;
    if (cudaMalloc(&p, kQueueSlots * 2 * sizeof(unsigned)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, kQueueSlots * 2 * sizeof(unsigned)) != cudaSuccess) return nullptr;
    g_queue_pool[d] = static_cast<unsigned*>(p);
  }
  const unsigned i = g_queue_next[d]++ % kQueueSlots;
  return g_queue_pool[d] + 2 * i;
}

unsigned long long wait_limit_ns() {
  static unsigned long long v = [] {
    const char* s = std::getenv("SPMM_WAIT_LIMIT_NS");
    unsigned long long x = s ? std::strtoull(s, nullptr, 10) : 0ull;
    return x ? x : 1000000000ull;  // one second
  }();
  return v;
}

namespace {
// Encoded tensor maps, reused across calls: an encoding depends only on its
// arguments, and repeated products on the same buffers are the common case.
struct MapKey {
  int rank, dt, swz;
  const void* base;
  uint64_t d0, d1, d2, s0, s1;
  uint32_t b0, b1, b2;
  bool operator==(const MapKey& o) const { return std::memcmp(this, &o, sizeof(MapKey)) == 0; }
};
struct MapEntry {
  MapKey k;
  CUtensorMap map;
};
constexpr int kMapCache = 128;
MapEntry g_maps[kMapCache];
int g_maps_used = 0, g_maps_next = 0;

bool map_lookup(const MapKey& k, CUtensorMap* out) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (int i = 0; i < g_maps_used; ++i)
    if (g_maps[i].k == k) {
      *out = g_maps[i].map;
      return true;
    }
  return false;
}
void map_store(const MapKey& k, const CUtensorMap& m) {
  std::lock_guard<std::mutex> lk(g_mu);
  MapEntry& e = g_maps[g_maps_next];
  e.k = k;
  e.map = m;
  g_maps_next = (g_maps_next + 1) % kMapCache;
  if (g_maps_used < kMapCache) ++g_maps_used;
}
MapKey map_key(int rank, int dt, int swz, const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t s0,
               uint64_t s1, uint32_t b0, uint32_t b1, uint32_t b2) {
  MapKey k;
  std::memset(&k, 0, sizeof(k));   // padding takes part in the comparison
  k.rank = rank;
  k.dt = dt;
  k.swz = swz;
  k.base = base;
  k.d0 = d0;
  k.d1 = d1;
  k.d2 = d2;
  k.s0 = s0;
  k.s1 = s1;
  k.b0 = b0;
  k.b1 = b1;
  k.b2 = b2;
  return k;
}
}  // namespace

spmm_status encode_tile_map_2d(CUtensorMap* map, CUtensorMapDataType dt, const void* base,
                               uint64_t inner, uint64_t outer, uint64_t row_stride_bytes,
                               uint32_t box_inner, uint32_t box_outer, CUtensorMapSwizzle swz) {
  const MapKey key = map_key(2, (int)dt, (int)swz, base, inner, outer, 0, row_stride_bytes, 0, box_inner,
                             box_outer, 0);
  if (map_lookup(key, map)) return SPMM_OK;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_encode) {
      cudaDriverEntryPointQueryResult q;
      void* fn = nullptr;
      cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                        cudaEnableDefault, &q);
      if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
        return fail(SPMM_ERR_CUDA, "cuTensorMapEncodeTiled entry point not available");
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
  }
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {row_stride_bytes};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, dt, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(SPMM_ERR_INVALID_ARG,
                "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) +
                    "): B needs a 16-byte aligned base and a row stride that is a multiple of 16 bytes");
  map_store(key, *map);
  return SPMM_OK;
}

spmm_status encode_panel_map_3d(CUtensorMap* map, const void* base, uint64_t N, uint64_t K,
                                uint64_t row_stride_bytes, uint32_t boxes, int elem_bytes) {
  if (elem_bytes != 1 && elem_bytes != 2) return fail(SPMM_ERR_UNSUPPORTED, "panel map: 8- or 16-bit elements");
  const uint64_t W = 128 / (uint64_t)elem_bytes;
  const CUtensorMapDataType dt = elem_bytes == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
  if (N % W || boxes == 0 || boxes > 256)
    return fail(SPMM_ERR_UNSUPPORTED, "panel map needs N to be a multiple of 128 bytes of columns");
  const MapKey key = map_key(3, (int)dt, (int)CU_TENSOR_MAP_SWIZZLE_128B, base, W, K, N / W, row_stride_bytes, 128,
                             (uint32_t)W, 16, boxes);
  if (map_lookup(key, map)) return SPMM_OK;
  CUtensorMap probe;
  spmm_status st = encode_tile_map_2d(&probe, dt, base, N, K, row_stride_bytes, (uint32_t)W, 16,
                                      CU_TENSOR_MAP_SWIZZLE_128B);   // resolves the entry point
  if (st != SPMM_OK) return st;
  cuuint64_t dims[3] = {W, K, N / W};
  cuuint64_t strides[2] = {row_stride_bytes, 128};
  cuuint32_t box[3] = {(cuuint32_t)W, 16, boxes};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(map, dt, 3, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(SPMM_ERR_UNSUPPORTED, "3-D panel tensor map rejected (" + std::to_string((int)r) + ")");
  map_store(key, *map);
  return SPMM_OK;
}

}  // namespace spmm

using namespace spmm;

extern "C" {

int spmm_abi_version(void) { return 1; }

const char* spmm_last_error(void) { return g_last_error.c_str(); }

int spmm_device_sm_count(void) { return sm_count(); }

spmm_status spmm_device_error_check(void* stream) {
  unsigned* w = device_error_word();
  if (!w) return fail(SPMM_ERR_CUDA, "no device error word");
  SPMM_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  unsigned v = 0;
  SPMM_CUDA_TRY(cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost));
  if (v) {
    SPMM_CUDA_TRY(cudaMemset(w, 0, sizeof(unsigned)));
    if (v == 64u)   // only the scale check fired: every wait completed
      return fail(SPMM_ERR_INVALID_ARG,
                  "an e4m3 block scale is not a positive normal power of two (the tcgen05 e4m3 kernels take "
                  "each scale as a UE8M0 exponent; spmm_quantize makes such scales)");
    return fail(SPMM_ERR_TIMEOUT, "a device-side pipeline wait timed out (code " + std::to_string(v) + ")");
  }
  return SPMM_OK;
}

spmm_status spmm_bcsr_mm(const spmm_bcsr_desc* A, const spmm_dense_desc* B, int N, float* C,
                         int ldc, const spmm_config* cfg, void* stream) {
  g_last_error.clear();
  if (!A || !B) return fail(SPMM_ERR_INVALID_ARG, "null descriptor");
  if (A->M < 0 || A->K < 0 || N < 0) return fail(SPMM_ERR_INVALID_ARG, "negative size");
  if (A->bC != 16) return fail(SPMM_ERR_UNSUPPORTED, "block width must be 16");
  if (A->bR != 16 && A->bR != 32 && A->bR != 64)
    return fail(SPMM_ERR_UNSUPPORTED, "block height must be 16, 32 or 64");
  if (A->M % A->bR) return fail(SPMM_ERR_INVALID_ARG, "M must be a multiple of the block height");
  if (A->K % 16) return fail(SPMM_ERR_INVALID_ARG, "K must be a multiple of 16");
  if (A->M == 0 || N == 0) return SPMM_OK;
  if (!A->row_ptr || !C || !B->data) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  // col_idx / vals may be NULL only when A stores no blocks (they are never read then)
  const bool e4m3 = A->dtype == SPMM_E4M3, split = A->dtype == SPMM_F16_SPLIT;
  if ((int)A->dtype < 0 || (int)A->dtype > 3) return fail(SPMM_ERR_INVALID_ARG, "unknown dtype");
  if (e4m3 && !A->scales) return fail(SPMM_ERR_INVALID_ARG, "E4M3 needs per-block scales");
  if (split && (!A->vals_lo || !B->data_lo))
    return fail(SPMM_ERR_INVALID_ARG, "F16_SPLIT needs the low halves of A and B");
  const int nmul = e4m3 ? 16 : 8;
  if (N % nmul) return fail(SPMM_ERR_UNSUPPORTED, "N must be a multiple of " + std::to_string(nmul));
  if (B->ldb < N || B->ldb % nmul) return fail(SPMM_ERR_MISALIGNED, "ldb must be >= N and a multiple of " + std::to_string(nmul));
  if (ldc < N || ldc % 4) return fail(SPMM_ERR_MISALIGNED, "ldc must be >= N and a multiple of 4");
  if (!aligned(A->vals, 16) || !aligned(B->data, 16) || !aligned(C, 16) ||
      (split && (!aligned(A->vals_lo, 16) || !aligned(B->data_lo, 16))))
    return fail(SPMM_ERR_MISALIGNED, "A values, B and C must be 16-byte aligned");
  if (A->K == 0) {
    // No block columns: C = 0 for the window.
    SPMM_CUDA_TRY(cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, A->M,
                                    static_cast<cudaStream_t>(stream)));
    return SPMM_OK;
  }
  LaunchRequest r;
  r.A = A;
  r.B = B;
  r.N = N;
  r.C = C;
  r.ldc = ldc;
  std::memset(&r.cfg, 0, sizeof(r.cfg));
  if (cfg) r.cfg = *cfg;
  r.stream = static_cast<cudaStream_t>(stream);
  if (r.cfg.kernel == 3) return launch_tc64(r);
  // kernel 0: tcgen05 for 64-row blocks (not e4m3, whose tcgen05 kernels need
  // power-of-two block scales), mma.sync otherwise
  if (r.cfg.kernel == 2 || (r.cfg.kernel == 0 && A->bR == 64 && !e4m3)) {
    spmm_status st = launch_tc(r);
    if (st != SPMM_ERR_UNSUPPORTED || r.cfg.kernel == 2) return st;
    g_last_error.clear();
  }
  return launch_mma(r);
}

spmm_status spmm_hcsr_mm(const spmm_bcsr_desc* A, const spmm_csr_desc* R, const spmm_dense_desc* B, int N,
                         float* C, int ldc, const spmm_config* cfg, void* stream) {
  g_last_error.clear();
  if (!A || !R || !B) return fail(SPMM_ERR_INVALID_ARG, "null descriptor");
  if (A->dtype != SPMM_F16) return fail(SPMM_ERR_UNSUPPORTED, "the hybrid product is fp16");
  if (R->M != A->M || R->K != A->K) return fail(SPMM_ERR_INVALID_ARG, "the two parts must have the same shape");
  if (A->M > 0 && !R->row_ptr) return fail(SPMM_ERR_INVALID_ARG, "null CSR row_ptr");
  spmm_config c;
  std::memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if (c.kernel != 0 && c.kernel != 2) return fail(SPMM_ERR_UNSUPPORTED, "the hybrid product runs on kernel 2");
  if (c.split_k > 1) return fail(SPMM_ERR_UNSUPPORTED, "the hybrid product has no split-K");
  c.kernel = 2;
  // the same argument checks as the BCSR product, then the launch with the CSR part
  if (A->M < 0 || A->K < 0 || N < 0) return fail(SPMM_ERR_INVALID_ARG, "negative size");
  if (A->bC != 16 || (A->bR != 16 && A->bR != 32 && A->bR != 64))
    return fail(SPMM_ERR_UNSUPPORTED, "block shape must be 16, 32 or 64 x 16");
  if (A->M % A->bR || A->K % 16) return fail(SPMM_ERR_INVALID_ARG, "M / K not multiples of the block shape");
  if (A->M == 0 || N == 0) return SPMM_OK;
  if (!A->row_ptr || !C || !B->data) return fail(SPMM_ERR_INVALID_ARG, "null pointer");
  if (N % 8) return fail(SPMM_ERR_UNSUPPORTED, "N must be a multiple of 8");
  if (B->ldb < N || B->ldb % 8) return fail(SPMM_ERR_MISALIGNED, "ldb must be >= N and a multiple of 8");
  if (ldc < N || ldc % 4) return fail(SPMM_ERR_MISALIGNED, "ldc must be >= N and a multiple of 4");
  if (!aligned(A->vals, 16) || !aligned(B->data, 16) || !aligned(C, 16))
    return fail(SPMM_ERR_MISALIGNED, "A values, B and C must be 16-byte aligned");
  if (A->K == 0) {
    SPMM_CUDA_TRY(cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, A->M, static_cast<cudaStream_t>(stream)));
    return SPMM_OK;
  }
  LaunchRequest r;
  r.A = A;
  r.B = B;
  r.N = N;
  r.C = C;
  r.ldc = ldc;
  r.cfg = c;
  r.stream = static_cast<cudaStream_t>(stream);
  r.csr = R;
  return launch_tc(r);
}

static spmm_status ref_launch(int bR, const int* hdr, const int* idx, const void* data,
                              const void* B, float* C, unsigned M, unsigned N, unsigned K,
                              void* stream) {
  spmm_bcsr_desc a;
  std::memset(&a, 0, sizeof(a));
  a.M = (int)M;
  a.K = (int)K;
  a.bR = bR;
  a.bC = 16;
  a.row_ptr = hdr;
  a.col_idx = idx;
  a.vals = data;
  a.dtype = SPMM_F16;
  spmm_dense_desc b;
  std::memset(&b, 0, sizeof(b));
  b.data = B;
  b.scale = 1.0f;
  b.ldb = (int)N;
  return spmm_bcsr_mm(&a, &b, (int)N, C, (int)N, nullptr, stream);
}

spmm_status sparseMatrixMulTensor_launch(const int* hdr, const int* idx, const void* data,
                                         const void* B, float* C, unsigned M, unsigned N,
                                         unsigned K, void* stream) {
  return ref_launch(16, hdr, idx, data, B, C, M, N, K, stream);
}
spmm_status sparseMatrixMulTensor32x16_launch(const int* hdr, const int* idx, const void* data,
                                              const void* B, float* C, unsigned M, unsigned N,
                                              unsigned K, void* stream) {
  return ref_launch(32, hdr, idx, data, B, C, M, N, K, stream);
}
spmm_status sparseMatrixMulTensor64x16_launch(const int* hdr, const int* idx, const void* data,
                                              const void* B, float* C, unsigned M, unsigned N,
                                              unsigned K, void* stream) {
  return ref_launch(64, hdr, idx, data, B, C, M, N, K, stream);
}
// The reference's variant kernels (src/cuda_kernels.cuh:47-99) compute the
// same product as the kernel of their block shape with another warp split or
// staging; each name launches this library's pipeline for that block shape.
#define SPMM_VARIANT_LAUNCHER(NAME, BR)                                                                   \
  spmm_status NAME(const int* hdr, const int* idx, const void* data, const void* B, float* C, unsigned M, \
                   unsigned N, unsigned K, void* stream) {                                                \
    return ref_launch(BR, hdr, idx, data, B, C, M, N, K, stream);                                         \
  }
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor_v2_launch, 16)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor_v3_launch, 16)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor_v1_improved_launch, 16)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor32x16_v2_launch, 32)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor32x16_shared_launch, 32)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor32x16_shared_vectorized_launch, 32)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor32x16_v2_shared_vectorized_launch, 32)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor64x16_v2_launch, 64)
SPMM_VARIANT_LAUNCHER(sparseMatrixMulTensor_option2_ldmatrix_sm80_launch, 16)
#undef SPMM_VARIANT_LAUNCHER
// sparseMatrixMulTensor1 (src/cuda_kernels.cu:330-355) multiplies square n x n
// matrices: its one size argument is M, N and K at once.
spmm_status sparseMatrixMulTensor1_launch(const int* hdr, const int* idx, const void* data, const void* B, float* C,
                                          unsigned n, void* stream) {
  return ref_launch(16, hdr, idx, data, B, C, n, n, n, stream);
}
spmm_status sparseMatrixMulTensorAdaptive_launch(const int* hdr, const int* idx, const void* data,
                                                 const void* B, float* C, unsigned M, unsigned N,
                                                 unsigned colBlocksPerRow, unsigned K,
                                                 void* stream) {
  (void)colBlocksPerRow;
  return ref_launch(16, hdr, idx, data, B, C, M, N, K, stream);
}
spmm_status sparseMatrixMulTensorAdaptive32x16_launch(const int* hdr, const int* idx,
                                                      const void* data, const void* B, float* C,
                                                      unsigned M, unsigned N,
                                                      unsigned colBlocksPerRow, unsigned K,
                                                      void* stream) {
  (void)colBlocksPerRow;
  return ref_launch(32, hdr, idx, data, B, C, M, N, K, stream);
}
spmm_status sparseMatrixMulTensorAdaptive64x16_launch(const int* hdr, const int* idx,
                                                      const void* data, const void* B, float* C,
                                                      unsigned M, unsigned N,
                                                      unsigned colBlocksPerRow, unsigned K,
                                                      void* stream) {
  (void)colBlocksPerRow;
  return ref_launch(64, hdr, idx, data, B, C, M, N, K, stream);
}

}  // extern "C"
