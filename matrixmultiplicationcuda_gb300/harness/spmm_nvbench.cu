// spmm_nvbench: NVBench-style benchmark harness for libbcsr_spmm.
//
// The reference measures its kernels with NVBench (nvbench_main.cu:326-1449:
// one bench_* function per kernel, axes over sizes / sparsity / pattern, a
// post-run check against the host multiply). This harness keeps that shape
// for the library's C ABI: named benches with axes, every state measured on a
// cold L2 (a 256 MB write before each sample) with CUDA events, samples taken
// until at least --min-samples and --min-time (or --max-time) are reached,
// the mean reported with its noise (relative standard deviation) as NVBench
// does (the event clock advances in ~2 us steps here, which the mean averages
// out and a median would not; the median is in the CSV / JSON too), and a
// post-run check of sampled block rows against an FP64 host product of the
// values the GPU multiplied. Throughput is TFLOP/s over nonzero-block FLOPs,
// algorithmic GB/s, and the fraction of the roofline
//   t_roof = max(FLOPs / tensor peak, compulsory bytes / HBM peak).
//
//   spmm_nvbench [--preset c1|c2|c3|c4|launch|compare|hybrid|all] [--tuning default,model,plan,sweep]
//                [--min-samples 20] [--min-time 0.2] [--max-time 2]
//                [--csv FILE] [--json FILE] [--model FILE] [--peaks FILE]
//                [--filter SUBSTRING] [--no-check] [--flush write|clean]
//
// Presets (seeded synthetic inputs):
//   c1  A 1024^2, 16x16 blocks, the reference generator's blockrandom pattern
//       at 10 % (mg::generate_matrix, seed 123), B = generate_matrix(1024,
//       1024, 0, "random", 16, 456); converted to BCSR on the GPU.
//   c2  A 8192^2 with 16x16, 32x16, 64x16 blocks; random, band (half-width 8
//       block columns), block-diagonal (256 x 256 dense tiles), log-normal
//       clustered (CV 1.5) patterns; 1 / 5 / 20 % block density; N 256, 1024,
//       4096; uniform[-1, 1] values.
//   c3  A 16384^2, 64x16 blocks, random 2 %, values N(0,1) x 10^U[-3,3] per
//       block; B 16384 x 512 N(0,1); fp16, bf16, e4m3 and split fp16.
//   c4  64 uneven products (M = K in [512, 8192], bR in {16, 32, 64},
//       random / band / block-diagonal, density log-uniform 0.5-25 %, N in
//       {128, 256, 512}): one persistent launch replayed from a CUDA graph
//       against 64 sequential launches, eager and graph-captured.
//   launch  host time per call and back-to-back launch rate (L2 warm) on the
//       c1 and c3 products (not part of "all").
//   compare the same product as BCSR, CSR (native kernel), dense through the
//       BCSR pipeline with every block stored, the native dense GEMM, and
//       cuBLAS GemmEx.
//   hybrid  the hybrid BCSR + CSR product across density thresholds.
//
// --flush clean: after the 256 MB write, read a second 256 MB buffer through
// L2 before each sample. The write alone leaves L2 full of dirty lines, and
// the timed launch pays for writing them back (~2 us on an empty kernel here);
// after the read L2 holds clean lines and the launch is cold without that.
//
// Tunings: default (the library's choice), model (the cost model's pick from
// the tuner table; a plan entry is built once and its runs are timed), plan
// (each per-matrix plan entry of the tuner table, the fastest reported),
// sweep (the exhaustive cold sweep's best).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "bcsr_spmm.h"
#include "bcsr_spmm_host.h"

namespace {

#define CK(x)                                                                               \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) {                                                                \
      std::fprintf(stderr, "CUDA error %s at %s:%d: %s\n", cudaGetErrorString(e_), __FILE__, \
                   __LINE__, #x);                                                           \
      std::exit(2);                                                                         \
    }                                                                                       \
  } while (0)
#define SK(x)                                                                                   \
  do {                                                                                          \
    spmm_status s_ = (x);                                                                       \
    if (s_ != SPMM_OK) {                                                                        \
      std::fprintf(stderr, "spmm error %d at %s:%d: %s (%s)\n", (int)s_, __FILE__, __LINE__, #x, \
                   spmm_last_error());                                                          \
      std::exit(3);                                                                             \
    }                                                                                           \
  } while (0)

struct Options {
  std::vector<std::string> presets{"c1", "c3", "c4"};
  std::vector<std::string> tunings{"default", "model"};
  int min_samples = 20;
  double min_time = 0.2, max_time = 2.0;
  std::string csv, json, model, peaks, filter;
  bool check = true;
  // cold-L2 method: false = write 256 MB before each sample (L2 is left full
  // of dirty lines, which the timed launch then writes back); true = the same
  // write, then a read of a second 256 MB buffer (L2 holds clean lines)
  bool clean_flush = false;
};

struct Peaks {
  double hbm_gbs = 6800, tflops = 1900;
  std::string source = "fallback";
};

std::string exe_dir() {
  char buf[4096];
  ssize_t n = readlink("/proc/self/exe", buf, sizeof(buf) - 1);
  if (n <= 0) return ".";
  buf[n] = 0;
  std::string s(buf);
  return s.substr(0, s.rfind('/'));
}

double json_number(const std::string& text, const std::string& key, double dflt) {
  size_t p = text.find("\"" + key + "\"");
  if (p == std::string::npos) return dflt;
  p = text.find(':', p);
  return p == std::string::npos ? dflt : std::atof(text.c_str() + p + 1);
}

Peaks load_peaks(const std::string& path) {
  Peaks pk;
  std::ifstream f(path);
  if (!f) return pk;
  std::stringstream ss;
  ss << f.rdbuf();
  pk.hbm_gbs = json_number(ss.str(), "hbm_gbs", pk.hbm_gbs);
  pk.tflops = json_number(ss.str(), "bf16_tflops", pk.tflops);
  pk.source = "measured";
  return pk;
}

const char* dtype_name(spmm_dtype d) {
  switch (d) {
    case SPMM_F16: return "f16";
    case SPMM_BF16: return "bf16";
    case SPMM_E4M3: return "e4m3";
    case SPMM_F16_SPLIT: return "f16_split";
  }
  return "?";
}
const char* pattern_name(int p) {
  static const char* n[] = {"random", "band", "blockdiag", "lognormal", "ref-blockrandom"};
  return p >= 0 && p <= 4 ? n[p] : "?";
}

std::string config_name(const spmm_config* c) {
  if (!c) return "library default";
  char b[128];
  if (c->kernel == 1)
    std::snprintf(b, sizeof(b), "mma nt%d st%d", c->n_tile, c->stages);
  else if (c->kernel == 3)
    std::snprintf(b, sizeof(b), "tc64 nt%d %s", c->n_tile, c->schedule ? "queue" : "static");
  else if (c->schedule == 2)
    std::snprintf(b, sizeof(b), "plan tc nt%d st%d acc%d", c->n_tile, c->stages, c->acc_buffers);
  else
    std::snprintf(b, sizeof(b), "tc nt%d st%d acc%d %s split%d", c->n_tile, c->stages, c->acc_buffers,
                  c->schedule ? "queue" : "static", c->split_k > 1 ? c->split_k : 1);
  return b;
}

// ---- one product on the device -----------------------------------------------------
struct Spec {
  std::string bench;
  int M, K, N, bR, pattern;   // pattern 4 = the reference generator's blockrandom
  double density, param;
  int value_dist, b_dist;
  spmm_dtype dtype;
  unsigned long long seed;
};

struct DeviceProduct {
  spmm_bcsr_desc A{};
  spmm_dense_desc B{};
  int N = 0;
  float* C = nullptr;
  long long nnzb = 0, cols_touched = 0;
  std::vector<int> rp, ci;
  std::vector<float> host_vals;   // the fp32 block values the product was built from
  std::vector<void*> owned;
  ~DeviceProduct() {
    for (void* p : owned) cudaFree(p);
  }
  template <class T>
  T* alloc(size_t bytes) {
    void* p = nullptr;
    CK(cudaMalloc(&p, bytes < 256 ? 256 : bytes));
    owned.push_back(p);
    return static_cast<T*>(p);
  }
};

size_t elem_bytes(spmm_dtype d) { return d == SPMM_E4M3 ? 1 : 2; }

// Builds A (BCSR, quantised to spec.dtype on the device), B and C.
void build_product(const Spec& s, DeviceProduct& P) {
  const int MB = s.M / s.bR;
  std::vector<float> vals;
  std::vector<float> Bf((size_t)s.K * s.N);
  if (s.pattern == 4) {
    // the reference's pipeline: generate a dense matrix, convert it to BCSR
    std::vector<float> dense((size_t)s.M * s.K);
    if (spmm_generate_matrix(s.M, s.K, 1.0 - s.density, "blockrandom", 16, (unsigned)s.seed, dense.data()) != 0)
      std::exit(4);
    std::vector<__half> h(dense.size());
    for (size_t i = 0; i < dense.size(); ++i) h[i] = __float2half(dense[i]);
    __half* dA = P.alloc<__half>(h.size() * 2);
    CK(cudaMemcpy(dA, h.data(), h.size() * 2, cudaMemcpyHostToDevice));
    int* rp = P.alloc<int>(sizeof(int) * (MB + 1));
    long long nnzb = 0;
    SK(spmm_dense_to_bcsr_count(dA, s.M, s.K, s.K, s.bR, 16, rp, &nnzb, nullptr));
    int* ci = P.alloc<int>(sizeof(int) * std::max(nnzb, 1LL));
    __half* v = P.alloc<__half>(2 * std::max(nnzb, 1LL) * s.bR * 16);
    SK(spmm_dense_to_bcsr_fill(dA, s.M, s.K, s.K, s.bR, 16, rp, ci, v, nullptr));
    CK(cudaDeviceSynchronize());
    P.rp.resize(MB + 1);
    P.ci.resize(nnzb);
    CK(cudaMemcpy(P.rp.data(), rp, sizeof(int) * (MB + 1), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(P.ci.data(), ci, sizeof(int) * nnzb, cudaMemcpyDeviceToHost));
    vals.resize((size_t)nnzb * s.bR * 16);
    std::vector<__half> hv(vals.size());
    CK(cudaMemcpy(hv.data(), v, hv.size() * 2, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < vals.size(); ++i) vals[i] = __half2float(hv[i]);
    if (spmm_generate_matrix(s.K, s.N, 0.0, "random", 16, 456u, Bf.data()) != 0) std::exit(4);
  } else {
    P.rp.resize(MB + 1);
    P.ci.resize((size_t)MB * (s.K / 16) + 1);
    const long long nnzb = spmm_gen_structure(s.M, s.K, s.bR, s.pattern, s.density, s.param, s.seed,
                                              P.rp.data(), P.ci.data());
    if (nnzb < 0) std::exit(4);
    P.ci.resize(nnzb);
    vals.resize((size_t)nnzb * s.bR * 16);
    spmm_gen_values(nnzb, s.bR, 16, s.value_dist, s.seed + 1, vals.data());
    spmm_gen_dense((long long)Bf.size(), s.b_dist, s.seed + 2, Bf.data());
  }
  P.nnzb = (long long)P.ci.size();
  P.cols_touched = (long long)std::set<int>(P.ci.begin(), P.ci.end()).size();
  const size_t nv = std::max<size_t>(vals.size(), 1);
  float* v32 = P.alloc<float>(nv * 4);
  float* b32 = P.alloc<float>(Bf.size() * 4);
  CK(cudaMemcpy(v32, vals.data(), vals.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b32, Bf.data(), Bf.size() * 4, cudaMemcpyHostToDevice));
  int* rp = P.alloc<int>(sizeof(int) * (MB + 1));
  int* ci = P.alloc<int>(sizeof(int) * std::max<long long>(P.nnzb, 1));
  CK(cudaMemcpy(rp, P.rp.data(), sizeof(int) * (MB + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ci, P.ci.data(), sizeof(int) * P.nnzb, cudaMemcpyHostToDevice));
  const size_t eb = elem_bytes(s.dtype);
  void* qa = P.alloc<void>(nv * eb);
  void* qa_lo = s.dtype == SPMM_F16_SPLIT ? P.alloc<void>(nv * 2) : nullptr;
  float* sa = s.dtype == SPMM_E4M3 ? P.alloc<float>(sizeof(float) * std::max<long long>(P.nnzb, 1)) : nullptr;
  void* qb = P.alloc<void>(Bf.size() * eb);
  void* qb_lo = s.dtype == SPMM_F16_SPLIT ? P.alloc<void>(Bf.size() * 2) : nullptr;
  float* sb = s.dtype == SPMM_E4M3 ? P.alloc<float>(sizeof(float)) : nullptr;
  if (!vals.empty()) SK(spmm_quantize(v32, vals.size(), s.dtype, s.bR * 16, qa, qa_lo, sa, nullptr));
  SK(spmm_quantize(b32, Bf.size(), s.dtype, (int)Bf.size(), qb, qb_lo, sb, nullptr));
  float bscale = 1.f;
  if (sb) CK(cudaMemcpy(&bscale, sb, 4, cudaMemcpyDeviceToHost));
  P.A.M = s.M;
  P.A.K = s.K;
  P.A.bR = s.bR;
  P.A.bC = 16;
  P.A.row_ptr = rp;
  P.A.col_idx = ci;
  P.A.vals = qa;
  P.A.vals_lo = qa_lo;
  P.A.scales = sa;
  P.A.dtype = s.dtype;
  P.B.data = qb;
  P.B.data_lo = qb_lo;
  P.B.scale = bscale;
  P.B.ldb = s.N;
  P.N = s.N;
  P.C = P.alloc<float>((size_t)s.M * s.N * 4);
  P.host_vals = std::move(vals);
}

// Value of stored element i of a quantised array as the GPU reads it.
double stored_value(const std::vector<uint8_t>& raw, const std::vector<uint8_t>& lo, spmm_dtype d, size_t i) {
  switch (d) {
    case SPMM_F16: return __half2float(reinterpret_cast<const __half*>(raw.data())[i]);
    case SPMM_BF16: return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(raw.data())[i]);
    case SPMM_E4M3: {
      __nv_fp8_e4m3 x;
      x.__x = raw[i];
      return (double)(float)x;
    }
    case SPMM_F16_SPLIT:
      return (double)__half2float(reinterpret_cast<const __half*>(raw.data())[i]) +
             (double)__half2float(reinterpret_cast<const __half*>(lo.data())[i]);
  }
  return 0;
}

// max |C - R| / max |R| over up to `rows` block rows (first, middle, last ...).
double check_rows(const DeviceProduct& P, int nrows) {
  const spmm_dtype d = P.A.dtype;
  const size_t eb = elem_bytes(d), K = P.A.K, N = P.N;
  const size_t nv = (size_t)P.nnzb * P.A.bR * 16;
  std::vector<uint8_t> a(nv * eb), alo, b(K * N * eb), blo;
  if (nv) CK(cudaMemcpy(a.data(), P.A.vals, a.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(b.data(), P.B.data, b.size(), cudaMemcpyDeviceToHost));
  if (d == SPMM_F16_SPLIT) {
    alo.resize(nv * 2);
    blo.resize(K * N * 2);
    if (nv) CK(cudaMemcpy(alo.data(), P.A.vals_lo, alo.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(blo.data(), P.B.data_lo, blo.size(), cudaMemcpyDeviceToHost));
  }
  std::vector<float> scales;
  if (d == SPMM_E4M3 && P.nnzb) {
    scales.resize(P.nnzb);
    CK(cudaMemcpy(scales.data(), P.A.scales, 4 * P.nnzb, cudaMemcpyDeviceToHost));
  }
  const int MB = P.A.M / P.A.bR, bR = P.A.bR;
  std::vector<int> rows;
  for (int k = 0; k < nrows; ++k) rows.push_back((int)((long long)k * (MB - 1) / std::max(nrows - 1, 1)));
  double md = 0, mr = 0;
  std::vector<double> R((size_t)bR * N);
  std::vector<float> C((size_t)bR * N);
  for (int br : rows) {
    std::fill(R.begin(), R.end(), 0.0);
    for (int j = P.rp[br]; j < P.rp[br + 1]; ++j) {
      const double sc = d == SPMM_E4M3 ? scales[j] * P.B.scale : 1.0;
      for (int r = 0; r < bR; ++r)
        for (int c = 0; c < 16; ++c) {
          const double av = stored_value(a, alo, d, (size_t)j * bR * 16 + r * 16 + c) * sc;
          if (av == 0) continue;
          const size_t krow = (size_t)P.ci[j] * 16 + c;
          for (size_t n = 0; n < N; ++n) R[r * N + n] += av * stored_value(b, blo, d, krow * N + n);
        }
    }
    CK(cudaMemcpy(C.data(), P.C + (size_t)br * bR * N, C.size() * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < R.size(); ++i) {
      md = std::max(md, std::fabs(C[i] - R[i]));
      mr = std::max(mr, std::fabs(R[i]));
    }
  }
  return mr > 0 ? md / mr : md;
}

// ---- measurement ---------------------------------------------------------------------
struct Sample {
  double median_us = 0, mean_us = 0, noise = 0;
  int samples = 0;
};

// Reads n 16-byte words through L2 (the clean flush's second pass).
__global__ void k_read_through_l2(const int4* __restrict__ p, size_t n, int* sink) {
  int acc = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int4 v = __ldcg(p + i);
    acc ^= v.x ^ v.w;
  }
  if (acc == 0x7fffffff) *sink = acc;   // keeps the loads; the flush buffer never holds this
}

__global__ void k_empty_launch() {}

struct Timer {
  cudaEvent_t e0, e1;
  void* flush = nullptr;
  void* flush2 = nullptr;
  int* sink = nullptr;
  size_t flush_bytes = 256u << 20;
  Timer() {
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaMalloc(&flush, flush_bytes));
  }
  ~Timer() {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(flush);
    cudaFree(flush2);
    cudaFree(sink);
  }
  void flush_l2(bool clean, int k) {
    CK(cudaMemsetAsync(flush, k & 0xff, flush_bytes, nullptr));
    if (!clean) return;
    if (!flush2) {
      CK(cudaMalloc(&flush2, flush_bytes));
      CK(cudaMemset(flush2, 0, flush_bytes));
      CK(cudaMalloc(&sink, sizeof(int)));
    }
    k_read_through_l2<<<1216, 256>>>(static_cast<const int4*>(flush2), flush_bytes / 16, sink);
    CK(cudaGetLastError());
  }
  template <class F>
  Sample measure(F&& run, const Options& o) {
    for (int w = 0; w < 3; ++w) run();
    CK(cudaDeviceSynchronize());
    std::vector<double> t;
    double total = 0;
    for (int k = 0;; ++k) {
      flush_l2(o.clean_flush, k);
      CK(cudaEventRecord(e0, nullptr));
      run();
      CK(cudaEventRecord(e1, nullptr));
      CK(cudaEventSynchronize(e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      t.push_back(ms * 1e3);
      total += ms * 1e-3;
      const int n = (int)t.size();
      if (n >= o.min_samples && (total >= o.min_time || n >= 2000)) break;
      if (total >= o.max_time && n >= 5) break;
    }
    Sample s;
    s.samples = (int)t.size();
    double sum = 0, sq = 0;
    for (double x : t) sum += x;
    s.mean_us = sum / t.size();
    for (double x : t) sq += (x - s.mean_us) * (x - s.mean_us);
    s.noise = t.size() > 1 ? std::sqrt(sq / (t.size() - 1)) / s.mean_us : 0;
    std::sort(t.begin(), t.end());
    s.median_us = t[t.size() / 2];
    return s;
  }
};

struct Row {
  Spec spec;
  std::string tuning, config;
  Sample s;
  double flops, bytes, tflops, gbs, roof_frac, rel_err;
  std::string bound;
  long long nnzb;
};

double algorithmic_bytes(const DeviceProduct& P) {
  const spmm_dtype d = P.A.dtype;
  const double eb = elem_bytes(d) * (d == SPMM_F16_SPLIT ? 2 : 1);
  return (double)P.nnzb * P.A.bR * 16 * eb + (d == SPMM_E4M3 ? 4.0 * P.nnzb : 0) + 4.0 * P.nnzb +
         4.0 * (P.A.M / P.A.bR + 1) + (double)P.cols_touched * 16 * P.N * eb + 4.0 * P.A.M * P.N;
}

void finish_row(Row& r, const DeviceProduct& P, const Peaks& pk) {
  r.nnzb = P.nnzb;
  r.flops = 2.0 * P.nnzb * P.A.bR * 16 * P.N;
  r.bytes = algorithmic_bytes(P);
  const double t = r.s.mean_us * 1e-6;
  r.tflops = r.flops / t / 1e12;
  r.gbs = r.bytes / t / 1e9;
  const double t_mem = r.bytes / (pk.hbm_gbs * 1e9), t_math = r.flops / (pk.tflops * 1e12);
  r.bound = t_mem >= t_math ? "hbm" : "tensor";
  r.roof_frac = std::max(t_mem, t_math) / t;
}

class Runner {
 public:
  Runner(const Options& o) : o_(o) {
    const std::string dir = exe_dir();
    pk_ = load_peaks(o.peaks.empty() ? dir + "/../../MEASURED_PEAKS.json" : o.peaks);
    const std::string mp = o.model.empty() ? dir + "/../data/costmodel.bin" : o.model;
    if (spmm_cost_model_load(mp.c_str(), &model_) != SPMM_OK) {
      std::fprintf(stderr, "no cost model (%s): model tuning falls back to the sweep\n", spmm_last_error());
      model_ = nullptr;
    }
  }
  Sample time_empty() {
    return timer_.measure([] { k_empty_launch<<<1, 32>>>(); }, o_);
  }
  ~Runner() {
    if (model_) spmm_cost_model_destroy(model_);
  }

  void product_bench(const Spec& spec) {
    std::string name = spec.bench + " M" + std::to_string(spec.M) + " N" + std::to_string(spec.N) + " bR" +
                       std::to_string(spec.bR) + " " + pattern_name(spec.pattern) + " " + dtype_name(spec.dtype);
    if (!o_.filter.empty() && name.find(o_.filter) == std::string::npos) return;
    DeviceProduct P;
    build_product(spec, P);
    for (const std::string& tuning : o_.tunings) {
      spmm_config cfg{};
      const spmm_config* pc = nullptr;
      if (tuning == "model" && model_) {
        SK(spmm_cost_model_select(model_, &P.A, P.N, &cfg, nullptr, nullptr));
        pc = &cfg;
      } else if (tuning == "sweep" || (tuning == "model" && !model_)) {
        std::vector<float> ms(spmm_tune_config_count());
        SK(spmm_tune_sweep(&P.A, &P.B, P.N, P.C, P.N, 2, 5, timer_.flush, timer_.flush_bytes, ms.data(), nullptr));
        SK(spmm_tune_config((int)(std::min_element(ms.begin(), ms.end()) - ms.begin()), &cfg));
        pc = &cfg;
      }
      Row r;
      r.spec = spec;
      r.tuning = tuning;
      if (tuning == "plan") {
        // a per-matrix plan on each tcgen05 configuration of the tuner's table
        // without split-K (the plan brings its own work queue), each timed the
        // same way; the row is the fastest, and its product is the one checked
        spmm_bcsr_plan* best = nullptr;
        for (int i = 0; i < spmm_tune_config_count(); ++i) {
          spmm_config tc{};
          SK(spmm_tune_config(i, &tc));
          if (tc.kernel != 2 || tc.schedule != 2) continue;   // the table's plan entries
          spmm_bcsr_plan* plan = nullptr;
          if (spmm_bcsr_plan_create(&P.A, P.N, &tc, nullptr, &plan) != SPMM_OK) continue;   // no kernel for it
          const Sample smp = timer_.measure([&] { SK(spmm_bcsr_plan_run(plan, &P.A, &P.B, P.N, P.C, P.N, nullptr)); }, o_);
          if (!best || smp.mean_us < r.s.mean_us) {
            if (best) SK(spmm_bcsr_plan_destroy(best));
            best = plan;
            r.s = smp;
          } else {
            SK(spmm_bcsr_plan_destroy(plan));
          }
        }
        if (!best) continue;   // no tcgen05 kernel for this block height and type
        int items = 0, groups = 0;
        spmm_config pcfg{};
        SK(spmm_bcsr_plan_info(best, &items, &groups, &pcfg));
        r.config = "plan " + config_name(&pcfg) + " (" + std::to_string(groups) + " rows split)";
        SK(spmm_bcsr_plan_run(best, &P.A, &P.B, P.N, P.C, P.N, nullptr));
        SK(spmm_bcsr_plan_destroy(best));
      } else if (pc && pc->kernel == 2 && pc->schedule == 2) {
        // a plan entry (the cost model's or the sweep's pick): build its plan
        // once, time its runs
        spmm_bcsr_plan* plan = nullptr;
        SK(spmm_bcsr_plan_create(&P.A, P.N, pc, nullptr, &plan));
        r.config = config_name(pc);
        r.s = timer_.measure([&] { SK(spmm_bcsr_plan_run(plan, &P.A, &P.B, P.N, P.C, P.N, nullptr)); }, o_);
        SK(spmm_bcsr_plan_destroy(plan));
      } else {
        r.config = config_name(pc);
        r.s = timer_.measure([&] { SK(spmm_bcsr_mm(&P.A, &P.B, P.N, P.C, P.N, pc, nullptr)); }, o_);
      }
      SK(spmm_device_error_check(nullptr));
      r.rel_err = o_.check ? check_rows(P, 2) : NAN;
      finish_row(r, P, pk_);
      rows_.push_back(r);
      print_row(r);
    }
  }

  void batched_bench() {
    // 64 products drawn (seeded) from the uneven workload's distributions
    std::mt19937_64 rng(2024);
    std::uniform_int_distribution<int> dm(512, 8192), d3(0, 2);
    std::uniform_real_distribution<double> du(std::log(0.005), std::log(0.25));
    const int bRs[3] = {16, 32, 64}, Ns[3] = {128, 256, 512};
    std::vector<std::unique_ptr<DeviceProduct>> probs;
    std::vector<spmm_problem> table;
    double flops = 0, bytes = 0;
    for (int i = 0; i < 64; ++i) {
      Spec s{};
      s.bench = "c4";
      s.M = s.K = std::min(8192, std::max(512, (int)std::lround(dm(rng) / 64.0) * 64));
      s.bR = bRs[d3(rng)];
      s.pattern = d3(rng);
      s.density = std::exp(du(rng));
      s.N = Ns[d3(rng)];
      const int KB = s.K / 16;
      s.param = s.pattern == 1 ? std::max(1.0, std::ceil(s.density * KB / 2))
                : s.pattern == 2 ? std::max(64.0, std::round(s.density * s.K / 64) * 64) : 0.0;
      s.value_dist = 0;
      s.b_dist = 0;
      s.dtype = SPMM_F16;
      s.seed = 2024000ull + i;
      probs.emplace_back(new DeviceProduct());
      build_product(s, *probs.back());
      DeviceProduct& P = *probs.back();
      spmm_problem pb{};
      pb.A = P.A;
      pb.B = P.B;
      pb.N = P.N;
      pb.C = P.C;
      pb.ldc = P.N;
      table.push_back(pb);
      flops += 2.0 * P.nnzb * P.A.bR * 16 * P.N;
      bytes += algorithmic_bytes(P);
    }
    spmm_batch_plan* plan = nullptr;
    SK(spmm_batch_plan_create(table.data(), (int)table.size(), nullptr, &plan));
    cudaStream_t cs;
    CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    SK(spmm_batch_run(plan, cs));
    CK(cudaStreamSynchronize(cs));
    auto capture = [&](auto&& body) {
      cudaGraph_t g;
      cudaGraphExec_t ge;
      CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      body();
      CK(cudaStreamEndCapture(cs, &g));
      CK(cudaGraphInstantiate(&ge, g, 0));
      CK(cudaGraphDestroy(g));
      return ge;
    };
    auto seq = [&](cudaStream_t st) {
      for (auto& P : probs) SK(spmm_bcsr_mm(&P->A, &P->B, P->N, P->C, P->N, nullptr, st));
    };
    seq(cs);   // first calls (per-kernel attributes) before capture
    CK(cudaStreamSynchronize(cs));
    cudaGraphExec_t gb = capture([&] { SK(spmm_batch_run(plan, cs)); });
    cudaGraphExec_t gs = capture([&] { seq(cs); });
    struct V {
      const char* name;
      Sample s;
    } v[3];
    v[0] = {"batched, graph replay", timer_.measure([&] { CK(cudaGraphLaunch(gb, nullptr)); }, o_)};
    v[1] = {"64 sequential launches", timer_.measure([&] { seq(nullptr); }, o_)};
    v[2] = {"64 sequential, graph replay", timer_.measure([&] { CK(cudaGraphLaunch(gs, nullptr)); }, o_)};
    SK(spmm_device_error_check(nullptr));
    std::printf("\n## c4: 64 uneven products (%.2f GFLOP, %.1f MB compulsory)\n\n", flops / 1e9, bytes / 1e6);
    std::printf("| variant | Samples | GPU Time (mean) | Noise | TFLOP/s | GB/s | Roofline | vs sequential |\n");
    std::printf("|---|---|---|---|---|---|---|---|\n");
    for (auto& x : v) {
      const double t = x.s.mean_us * 1e-6;
      std::printf("| %s | %d | %.2f us | %.2f%% | %.1f | %.0f | %.3f | %.2fx |\n", x.name, x.s.samples, x.s.mean_us,
                  100 * x.s.noise, flops / t / 1e12, bytes / t / 1e9, (bytes / (pk_.hbm_gbs * 1e9)) / t,
                  v[1].s.mean_us / x.s.mean_us);
      batch_lines_.push_back({x.name, x.s.mean_us, flops, bytes});
    }
    std::fflush(stdout);
    cudaGraphExecDestroy(gb);
    cudaGraphExecDestroy(gs);
    cudaStreamDestroy(cs);
    spmm_batch_plan_destroy(plan);
  }

  // Host time per call and back-to-back launch rate (L2 warm: the same buffers
  // every launch; consecutive launches may overlap through programmatic
  // dependent launch unless SPMM_NO_PDL is set). plan_nt > 0: the calls are
  // spmm_bcsr_plan_run_ex on a per-matrix plan with that column tile and
  // `plan_acc` accumulators, with `flags` (SPMM_RUN_INPUTS_READY: nothing in
  // the loop writes A or B, so each launch starts while the one before drains C).
  void launch_bench(const Spec& spec, const char* label, int plan_nt = 0, unsigned flags = 0, int plan_acc = 1) {
    DeviceProduct P;
    build_product(spec, P);
    constexpr int kCalls = 200;
    spmm_bcsr_plan* plan = nullptr;
    if (plan_nt > 0) {
      spmm_config pc{};
      pc.kernel = 2;
      pc.n_tile = plan_nt;
      pc.acc_buffers = plan_acc;
      SK(spmm_bcsr_plan_create(&P.A, P.N, &pc, nullptr, &plan));
    }
    auto call = [&] {
      if (plan) SK(spmm_bcsr_plan_run_ex(plan, &P.A, &P.B, P.N, P.C, P.N, flags, nullptr));
      else SK(spmm_bcsr_mm(&P.A, &P.B, P.N, P.C, P.N, nullptr, nullptr));
    };
    for (int i = 0; i < 20; ++i) call();
    CK(cudaDeviceSynchronize());
    double host_us = 1e30, gpu_us = 1e30;
    for (int rep = 0; rep < 5; ++rep) {
      CK(cudaEventRecord(timer_.e0, nullptr));
      const auto t0 = std::chrono::steady_clock::now();
      for (int i = 0; i < kCalls; ++i) call();
      const auto t1 = std::chrono::steady_clock::now();
      CK(cudaEventRecord(timer_.e1, nullptr));
      CK(cudaEventSynchronize(timer_.e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, timer_.e0, timer_.e1));
      host_us = std::min(host_us, std::chrono::duration<double, std::micro>(t1 - t0).count() / kCalls);
      gpu_us = std::min(gpu_us, ms * 1e3 / kCalls);
    }
    std::printf("| %s | %s | %.2f us | %.2f us | %.1f |\n", label, std::getenv("SPMM_NO_PDL") ? "off" : "on", host_us,
                gpu_us, 2.0 * P.nnzb * P.A.bR * 16 * P.N / (gpu_us * 1e-6) / 1e12);
    std::fflush(stdout);
    if (plan) SK(spmm_bcsr_plan_destroy(plan));
  }

  // The same product as BCSR (cost-model configuration), as CSR (the native
  // CSR kernel), and densely: the BCSR pipeline with every block stored, the
  // native tcgen05 dense GEMM, and cuBLAS GemmEx (fp16 in, fp32 out) as the
  // library reference point.
  void compare_bench(const Spec& spec, const char* label) {
    DeviceProduct P;
    build_product(spec, P);
    const int M = spec.M, K = spec.K, N = spec.N, bR = spec.bR;
    // host CSR of the stored fp16 values, columns ascending
    std::vector<int> crp(M + 1, 0), cci;
    std::vector<__half> cv;
    for (int br = 0; br < M / bR; ++br)
      for (int r = 0; r < bR; ++r) {
        for (int j = P.rp[br]; j < P.rp[br + 1]; ++j)
          for (int c = 0; c < 16; ++c) {
            const __half h = __float2half(P.host_vals[((size_t)j * bR + r) * 16 + c]);
            if (__half2float(h) != 0.f) {
              cci.push_back(P.ci[j] * 16 + c);
              cv.push_back(h);
            }
          }
        crp[br * bR + r + 1] = (int)cci.size();
      }
    int* d_crp = P.alloc<int>(sizeof(int) * (M + 1));
    int* d_cci = P.alloc<int>(sizeof(int) * std::max<size_t>(cci.size(), 1));
    __half* d_cv = P.alloc<__half>(2 * std::max<size_t>(cv.size(), 1));
    CK(cudaMemcpy(d_crp, crp.data(), sizeof(int) * (M + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_cci, cci.data(), sizeof(int) * cci.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_cv, cv.data(), 2 * cv.size(), cudaMemcpyHostToDevice));
    spmm_csr_desc R{M, K, d_crp, d_cci, d_cv};
    // the whole matrix, densely: fp16 M x K, and as BCSR with every block stored
    std::vector<__half> dense((size_t)M * K, __float2half(0.f));
    for (int br = 0; br < M / bR; ++br)
      for (int j = P.rp[br]; j < P.rp[br + 1]; ++j)
        for (int r = 0; r < bR; ++r)
          for (int c = 0; c < 16; ++c)
            dense[(size_t)(br * bR + r) * K + P.ci[j] * 16 + c] = __float2half(P.host_vals[((size_t)j * bR + r) * 16 + c]);
    __half* d_dense = P.alloc<__half>(dense.size() * 2);
    CK(cudaMemcpy(d_dense, dense.data(), dense.size() * 2, cudaMemcpyHostToDevice));
    const int MB = M / bR, KB = K / 16;
    std::vector<int> frp(MB + 1), fci((size_t)MB * KB);
    std::vector<__half> fv((size_t)M * K);
    for (int br = 0; br < MB; ++br) {
      frp[br] = br * KB;
      for (int j = 0; j < KB; ++j) {
        fci[(size_t)br * KB + j] = j;
        for (int r = 0; r < bR; ++r)
          std::memcpy(&fv[(((size_t)br * KB + j) * bR + r) * 16], &dense[(size_t)(br * bR + r) * K + j * 16], 32);
      }
    }
    frp[MB] = MB * KB;
    int* d_frp = P.alloc<int>(sizeof(int) * (MB + 1));
    int* d_fci = P.alloc<int>(sizeof(int) * fci.size());
    __half* d_fv = P.alloc<__half>(fv.size() * 2);
    CK(cudaMemcpy(d_frp, frp.data(), sizeof(int) * (MB + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_fci, fci.data(), sizeof(int) * fci.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_fv, fv.data(), fv.size() * 2, cudaMemcpyHostToDevice));
    spmm_bcsr_desc F = P.A;
    F.row_ptr = d_frp;
    F.col_idx = d_fci;
    F.vals = d_fv;
    spmm_config cs{}, cf{};
    const spmm_config* pcs = nullptr;
    const spmm_config* pcf = nullptr;
    if (model_) {
      SK(spmm_cost_model_select(model_, &P.A, N, &cs, nullptr, nullptr));
      SK(spmm_cost_model_select(model_, &F, N, &cf, nullptr, nullptr));
      pcs = &cs;
      pcf = &cf;
    }
    cublasHandle_t hb;
    if (cublasCreate(&hb) != CUBLAS_STATUS_SUCCESS) std::exit(5);
    const float one = 1.f, zero = 0.f;
    struct V {
      std::string name;
      Sample s;
    };
    std::vector<V> v;
    v.push_back({"BCSR " + config_name(pcs), timer_.measure([&] { SK(spmm_bcsr_mm(&P.A, &P.B, N, P.C, N, pcs, nullptr)); }, o_)});
    v.push_back({"CSR (native kernel)", timer_.measure([&] { SK(spmm_csr_mm(&R, &P.B, N, P.C, N, nullptr)); }, o_)});
    v.push_back({"dense: BCSR pipeline, all blocks, " + config_name(pcf),
                 timer_.measure([&] { SK(spmm_bcsr_mm(&F, &P.B, N, P.C, N, pcf, nullptr)); }, o_)});
    v.push_back({"dense: native tcgen05 GEMM (spmm_dense_mm)", timer_.measure([&] {
                   SK(spmm_dense_mm(d_dense, K, &P.B, M, K, N, SPMM_F16, P.C, N, nullptr));
                 }, o_)});
    v.push_back({"dense: cuBLAS GemmEx (library)", timer_.measure([&] {
                   cublasGemmEx(hb, CUBLAS_OP_N, CUBLAS_OP_N, N, M, K, &one, P.B.data, CUDA_R_16F, N, d_dense,
                                CUDA_R_16F, K, &zero, P.C, CUDA_R_32F, N, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
                 }, o_)});
    SK(spmm_device_error_check(nullptr));
    cublasDestroy(hb);
    const double useful = 2.0 * P.nnzb * bR * 16 * N, dense_fl = 2.0 * M * K * N;
    std::printf("\n## compare: %s (nnzb %lld, CSR nnz %zu)\n\n", label, P.nnzb, cci.size());
    std::printf("| method | Samples | GPU Time (mean) | Noise | TFLOP/s (nonzero blocks) | dense-equivalent TFLOP/s |\n");
    std::printf("|---|---|---|---|---|---|\n");
    for (auto& x : v)
      std::printf("| %s | %d | %.2f us | %.2f%% | %.1f | %.1f |\n", x.name.c_str(), x.s.samples, x.s.mean_us,
                  100 * x.s.noise, useful / (x.s.mean_us * 1e-6) / 1e12, dense_fl / (x.s.mean_us * 1e-6) / 1e12);
    std::fflush(stdout);
  }

  // The hybrid product across thresholds, as the reference's CLI sweeps them
  // (main.cu:567-590), on a matrix with dense blocks and scattered entries.
  void hybrid_bench() {
    const int M = 4096, K = 4096, N = 1024;
    std::vector<float> blocks((size_t)M * K), scatter((size_t)M * K), B((size_t)K * N);
    if (spmm_generate_matrix(M, K, 0.9, "blockrandom", 16, 7u, blocks.data()) != 0 ||
        spmm_generate_matrix(M, K, 0.98, "random", 16, 8u, scatter.data()) != 0)
      std::exit(4);
    std::vector<__half> A((size_t)M * K);
    for (size_t i = 0; i < A.size(); ++i) A[i] = __float2half(blocks[i] != 0.f ? blocks[i] : scatter[i]);
    spmm_gen_dense((long long)B.size(), 0, 9, B.data());
    std::vector<__half> Bh(B.size());
    for (size_t i = 0; i < B.size(); ++i) Bh[i] = __float2half(B[i]);
    DeviceProduct P;
    __half* dB = P.alloc<__half>(Bh.size() * 2);
    float* dC = P.alloc<float>((size_t)M * N * 4);
    CK(cudaMemcpy(dB, Bh.data(), Bh.size() * 2, cudaMemcpyHostToDevice));
    spmm_dense_desc Bd{dB, nullptr, 1.f, N};
    std::printf("\n## hybrid: A %dx%d (10%% dense 16x16 blocks + 2%% scattered entries), N %d, fp16\n\n", M, K, N);
    std::printf("| threshold | BCSR blocks | CSR entries | method | Samples | GPU Time (mean) | Noise | TFLOP/s (stored entries) |\n");
    std::printf("|---|---|---|---|---|---|---|---|\n");
    for (float th : {0.0f, 0.2f, 0.4f, 0.6f, 0.8f, 1.1f}) {
      long long nnzb = 0, nnz = 0;
      if (spmm_host_dense_to_hcsr(A.data(), M, K, th, &nnzb, &nnz, nullptr, nullptr, nullptr, nullptr, nullptr,
                                  nullptr) != 0)
        std::exit(4);
      std::vector<int> bh(M / 16 + 1), bi(std::max(nnzb, 1LL)), ch(M + 1), cx(std::max(nnz, 1LL));
      std::vector<__half> bd(std::max(nnzb, 1LL) * 256), cd(std::max(nnz, 1LL));
      spmm_host_dense_to_hcsr(A.data(), M, K, th, &nnzb, &nnz, bh.data(), bi.data(), bd.data(), ch.data(), cx.data(),
                              cd.data());
      DeviceProduct Q;
      int* d_bh = Q.alloc<int>(4 * bh.size());
      int* d_bi = Q.alloc<int>(4 * bi.size());
      __half* d_bd = Q.alloc<__half>(2 * bd.size());
      int* d_ch = Q.alloc<int>(4 * ch.size());
      int* d_cx = Q.alloc<int>(4 * cx.size());
      __half* d_cd = Q.alloc<__half>(2 * cd.size());
      CK(cudaMemcpy(d_bh, bh.data(), 4 * bh.size(), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(d_bi, bi.data(), 4 * bi.size(), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(d_bd, bd.data(), 2 * bd.size(), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(d_ch, ch.data(), 4 * ch.size(), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(d_cx, cx.data(), 4 * cx.size(), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(d_cd, cd.data(), 2 * cd.size(), cudaMemcpyHostToDevice));
      spmm_bcsr_desc Ab{M, K, 16, 16, d_bh, d_bi, d_bd, nullptr, nullptr, SPMM_F16};
      spmm_csr_desc R{M, K, d_ch, d_cx, d_cd};
      spmm_hcsr_plan* plan = nullptr;
      SK(spmm_hcsr_plan_create(&Ab, &R, nullptr, &plan));
      long long nblk = 0, ngat = 0;
      SK(spmm_hcsr_plan_info(plan, &nblk, &ngat));
      Sample se = timer_.measure([&] { SK(spmm_hcsr_mm(&Ab, &R, &Bd, N, dC, N, nullptr, nullptr)); }, o_);
      Sample sp = timer_.measure([&] { SK(spmm_hcsr_plan_run(plan, &Bd, N, dC, N, nullptr, nullptr)); }, o_);
      SK(spmm_device_error_check(nullptr));
      SK(spmm_hcsr_plan_destroy(plan));
      const double fl = 2.0 * ((double)nnzb * 256 + nnz) * N;
      std::printf("| %.1f | %lld | %lld | CSR pass in the epilogue | %d | %.2f us | %.2f%% | %.1f |\n", th, nnzb, nnz,
                  se.samples, se.mean_us, 100 * se.noise, fl / (se.mean_us * 1e-6) / 1e12);
      std::printf("| %.1f | %lld | %lld | planned: %lld gather blocks | %d | %.2f us | %.2f%% | %.1f |\n", th, nnzb,
                  nnz, ngat, sp.samples, sp.mean_us, 100 * sp.noise, fl / (sp.mean_us * 1e-6) / 1e12);
      std::fflush(stdout);
    }
  }

  void header(const char* title) {
    std::printf("\n## %s\n\n", title);
    std::printf("| M | N | bR | pattern | density | dtype | tuning | config | Samples | GPU Time (mean) | Noise | "
                "TFLOP/s | GB/s | Roofline | bound | max rel err |\n");
    std::printf("|---|---|---|---|---|---|---|---|---|---|---|---|---|---|---|---|\n");
    std::fflush(stdout);
  }

  void print_row(const Row& r) {
    std::printf("| %d | %d | %d | %s | %.3g | %s | %s | %s | %d | %.2f us | %.2f%% | %.1f | %.0f | %.3f | %s | %.2e |\n",
                r.spec.M, r.spec.N, r.spec.bR, pattern_name(r.spec.pattern), r.spec.density, dtype_name(r.spec.dtype),
                r.tuning.c_str(), r.config.c_str(), r.s.samples, r.s.mean_us, 100 * r.s.noise, r.tflops, r.gbs,
                r.roof_frac, r.bound.c_str(), r.rel_err);
    std::fflush(stdout);
  }

  void write_outputs() {
    if (!o_.csv.empty()) {
      FILE* f = std::fopen(o_.csv.c_str(), "w");
      if (f) {
        std::fprintf(f, "bench,M,K,N,bR,pattern,density,dtype,tuning,config,nnzb,samples,mean_us,median_us,noise,tflops,gbs,"
                        "roofline_frac,bound,max_rel_err\n");
        for (const Row& r : rows_)
          std::fprintf(f, "%s,%d,%d,%d,%d,%s,%g,%s,%s,%s,%lld,%d,%.4f,%.4f,%.5f,%.3f,%.1f,%.4f,%s,%.3e\n",
                       r.spec.bench.c_str(), r.spec.M, r.spec.K, r.spec.N, r.spec.bR, pattern_name(r.spec.pattern),
                       r.spec.density, dtype_name(r.spec.dtype), r.tuning.c_str(), r.config.c_str(), r.nnzb,
                       r.s.samples, r.s.mean_us, r.s.median_us, r.s.noise, r.tflops, r.gbs, r.roof_frac, r.bound.c_str(), r.rel_err);
        std::fclose(f);
      }
    }
    if (!o_.json.empty()) {
      FILE* f = std::fopen(o_.json.c_str(), "w");
      if (f) {
        std::fprintf(f, "{\"peaks\": {\"hbm_gbs\": %.1f, \"tflops\": %.1f, \"source\": \"%s\"}, \"states\": [\n",
                     pk_.hbm_gbs, pk_.tflops, pk_.source.c_str());
        for (size_t i = 0; i < rows_.size(); ++i) {
          const Row& r = rows_[i];
          std::fprintf(f,
                       " {\"bench\": \"%s\", \"M\": %d, \"N\": %d, \"bR\": %d, \"pattern\": \"%s\", \"density\": %g, "
                       "\"dtype\": \"%s\", \"tuning\": \"%s\", \"config\": \"%s\", \"nnzb\": %lld, \"mean_us\": %.4f, "
                       "\"median_us\": %.4f, "
                       "\"noise\": %.5f, \"tflops\": %.3f, \"gbs\": %.1f, \"roofline_frac\": %.4f, \"bound\": \"%s\", "
                       "\"max_rel_err\": %.3e}%s\n",
                       r.spec.bench.c_str(), r.spec.M, r.spec.N, r.spec.bR, pattern_name(r.spec.pattern), r.spec.density,
                       dtype_name(r.spec.dtype), r.tuning.c_str(), r.config.c_str(), r.nnzb, r.s.mean_us, r.s.median_us,
                       r.s.noise,
                       r.tflops, r.gbs, r.roof_frac, r.bound.c_str(), std::isnan(r.rel_err) ? -1.0 : r.rel_err,
                       i + 1 < rows_.size() ? "," : "");
        }
        std::fprintf(f, "], \"batched\": [\n");
        for (size_t i = 0; i < batch_lines_.size(); ++i)
          std::fprintf(f, " {\"variant\": \"%s\", \"mean_us\": %.3f, \"gflop\": %.4f, \"mb\": %.2f}%s\n",
                       batch_lines_[i].name.c_str(), batch_lines_[i].us, batch_lines_[i].flops / 1e9,
                       batch_lines_[i].bytes / 1e6, i + 1 < batch_lines_.size() ? "," : "");
        std::fprintf(f, "]}\n");
        std::fclose(f);
      }
    }
  }

  const Peaks& peaks() const { return pk_; }

 private:
  struct BatchLine {
    std::string name;
    double us, flops, bytes;
  };
  Options o_;
  Peaks pk_;
  spmm_cost_model* model_ = nullptr;
  Timer timer_;
  std::vector<Row> rows_;
  std::vector<BatchLine> batch_lines_;
};

std::vector<std::string> split(const std::string& s) {
  std::vector<std::string> out;
  std::stringstream ss(s);
  std::string x;
  while (std::getline(ss, x, ',')) out.push_back(x);
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "%s needs a value\n", a.c_str());
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "--preset") {
      std::string p = next();
      o.presets = p == "all" ? std::vector<std::string>{"c1", "c2", "c3", "c4"} : split(p);
    } else if (a == "--tuning") {
      o.tunings = split(next());
    } else if (a == "--min-samples") {
      o.min_samples = std::atoi(next().c_str());
    } else if (a == "--min-time") {
      o.min_time = std::atof(next().c_str());
    } else if (a == "--max-time") {
      o.max_time = std::atof(next().c_str());
    } else if (a == "--csv") {
      o.csv = next();
    } else if (a == "--json") {
      o.json = next();
    } else if (a == "--model") {
      o.model = next();
    } else if (a == "--peaks") {
      o.peaks = next();
    } else if (a == "--filter") {
      o.filter = next();
    } else if (a == "--no-check") {
      o.check = false;
    } else if (a == "--flush") {
      const std::string f = next();
      if (f != "write" && f != "clean") {
        std::fprintf(stderr, "--flush takes write or clean\n");
        return 1;
      }
      o.clean_flush = f == "clean";
    } else {
      std::fprintf(stderr, "usage: spmm_nvbench [--preset c1,c2,c3,c4|all] [--tuning default,model,plan,sweep] "
                           "[--min-samples N] [--min-time S] [--max-time S] [--csv F] [--json F] [--model F] "
                           "[--peaks F] [--filter S] [--no-check] [--flush write|clean]\n");
      return a == "--help" || a == "-h" ? 0 : 1;
    }
  }
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, 0));
  Runner run(o);
  std::printf("# spmm_nvbench on %s (%d SMs); peaks (%s): HBM %.0f GB/s, tensor %.0f TFLOP/s; cold L2 "
              "(256 MB written before each sample%s)\n",
              prop.name, prop.multiProcessorCount, run.peaks().source.c_str(), run.peaks().hbm_gbs, run.peaks().tflops,
              o.clean_flush ? ", then a second 256 MB buffer read, so L2 holds clean lines" : "");
  for (const std::string& p : o.presets) {
    if (p == "c1") {
      run.header("c1: A 1024^2, 16x16 blocks, reference blockrandom 10 %, N 1024");
      Spec s{"c1", 1024, 1024, 1024, 16, 4, 0.10, 0.0, 0, 0, SPMM_F16, 123};
      run.product_bench(s);
    } else if (p == "c2") {
      run.header("c2: A 8192^2 sweep (block shapes x patterns x densities x N), fp16");
      for (int bR : {16, 32, 64})
        for (int pat : {0, 1, 2, 3})
          for (double dens : {0.01, 0.05, 0.20}) {
            if (pat == 2 && dens != 0.01) continue;   // 256 x 256 dense tiles fix the density (3.1 %)
            for (int N : {256, 1024, 4096}) {
              const double param = pat == 1 ? 8.0 : pat == 2 ? 256.0 : pat == 3 ? 1.5 : 0.0;
              Spec s{"c2", 8192, 8192, N, bR, pat, pat == 2 ? 256.0 / 8192 : dens, param, 0, 0, SPMM_F16,
                     (unsigned long long)(1000 + bR * 100 + pat * 10 + (int)(dens * 100))};
              run.product_bench(s);
            }
          }
    } else if (p == "c3") {
      run.header("c3: A 16384^2, 64x16 blocks, random 2 %, N(0,1)*10^U[-3,3], N 512, four precisions");
      for (spmm_dtype d : {SPMM_F16, SPMM_BF16, SPMM_E4M3, SPMM_F16_SPLIT}) {
        Spec s{"c3", 16384, 16384, 512, 64, 0, 0.02, 0.0, 1, 2, d, 20240};
        run.product_bench(s);
      }
    } else if (p == "c4") {
      run.batched_bench();
    } else if (p == "compare") {
      run.compare_bench(Spec{"compare", 1024, 1024, 1024, 16, 4, 0.10, 0.0, 0, 0, SPMM_F16, 123},
                        "A 1024^2, 16x16 blocks, reference blockrandom 10 %, N 1024");
      run.compare_bench(Spec{"compare", 8192, 8192, 1024, 16, 0, 0.05, 0.0, 0, 0, SPMM_F16, 77},
                        "A 8192^2, 16x16 blocks, random 5 %, N 1024");
      run.compare_bench(Spec{"compare", 16384, 16384, 512, 64, 0, 0.02, 0.0, 1, 2, SPMM_F16, 20240},
                        "A 16384^2, 64x16 blocks, random 2 %, N 512");
    } else if (p == "hybrid") {
      run.hybrid_bench();
    } else if (p == "floor") {
      // the timing floor of this method: an empty kernel, measured like every row
      const Sample f = run.time_empty();
      std::printf("\n## floor: an empty kernel timed like every row\n\n| kernel | mean | median | samples |\n"
                  "|---|---|---|---|\n| empty, <<<1, 32>>> | %.2f us | %.2f us | %d |\n",
                  f.mean_us, f.median_us, f.samples);
    } else if (p == "launch") {
      std::printf("\n## launch: host time per call, back-to-back launches (L2 warm)\n\n");
      std::printf("| product | PDL | host per call | GPU per launch | TFLOP/s |\n|---|---|---|---|---|\n");
      const Spec c1{"launch", 1024, 1024, 1024, 16, 4, 0.10, 0.0, 0, 0, SPMM_F16, 123};
      run.launch_bench(c1, "1024^2 16x16 10%, N 1024, spmm_bcsr_mm");
      run.launch_bench(c1, "the same, plan (256 columns)", 256, 0u, 2);
      run.launch_bench(c1, "the same, plan (256 columns), SPMM_RUN_INPUTS_READY", 256, SPMM_RUN_INPUTS_READY, 2);
      const Spec c3{"launch", 16384, 16384, 512, 64, 0, 0.02, 0.0, 1, 2, SPMM_F16, 20240};
      run.launch_bench(c3, "16384^2 64x16 2%, N 512, spmm_bcsr_mm");
      run.launch_bench(c3, "the same, plan (512 columns)", 512, 0u);
      run.launch_bench(c3, "the same, plan (512 columns), SPMM_RUN_INPUTS_READY", 512, SPMM_RUN_INPUTS_READY);
    } else {
      std::fprintf(stderr, "unknown preset %s\n", p.c_str());
      return 1;
    }
  }
  run.write_outputs();
  return 0;
}
