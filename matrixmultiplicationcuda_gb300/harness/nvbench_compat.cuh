// nvbench_compat.cuh -- the part of NVBench's C++ surface that benchmark code
// for the BCSR path uses, so that benches written for NVBench compile and run
// here, where NVBench is not installed (the reference fetches it over the
// network at configure time, CMakeLists.txt:63-64).
//
// Written from NVBench's public documentation, keeping its names and meaning:
//   NVBENCH_BENCH(fn).set_name(s).add_int64_axis(name, {values})
//       .add_float64_axis / .add_string_axis / .set_min_samples / .set_timeout
//   state.get_int64 / get_float64 / get_string, state.add_element_count,
//   state.add_global_memory_reads<T> / _writes<T>, state.skip(reason),
//   state.get_summary(tag).set_string / remove_value,
//   state.exec(fn(launch&)) and state.exec(exec_tag::timer, fn(launch&, timer&))
//   with timer.start() / timer.stop(), launch.get_stream() (a cudaStream_t),
//   NVBENCH_MAIN, and the command line -b/--benchmark, -a/--axis "N=[32,64]",
//   --min-samples, --timeout, --csv FILE, --json FILE, -l/--list.
//
// Measurement is NVBench's "cold" one: before every sample the L2 is flushed
// (a write of twice its size) and the stream synchronised; a sample's GPU time
// is CUDA events around the launch (or around timer.start() / timer.stop()),
// its CPU time the host clock around the same span. Samples are taken until
// both the minimum count and the minimum time are reached (or the timeout).
// Summaries use NVBench's tags (nv/cold/time/gpu/mean, .../min, .../max,
// .../stdev/relative, nv/cold/time/cpu/..., nv/cold/sample_size,
// nv/element_count, nv/gmem/bw); min, max and the CPU times start hidden
// ("hide" set), as NVBench prints them, and a bench may show them with
// remove_value("hide"). Not provided: batch ("hot") measurements, type axes,
// multiple devices, throttling detection.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

namespace nvbench {

using int64_t = std::int64_t;
using float64_t = double;

namespace detail {
inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "nvbench: %s failed: %s\n", what, cudaGetErrorString(e));
    std::exit(2);
  }
}
}  // namespace detail

// A stream owned by one state; converts to cudaStream_t so it can go straight
// into a launch configuration or an API call.
class cuda_stream {
 public:
  cuda_stream() { detail::cuda_check(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "cudaStreamCreate"); }
  ~cuda_stream() { cudaStreamDestroy(s_); }
  cuda_stream(const cuda_stream&) = delete;
  cuda_stream& operator=(const cuda_stream&) = delete;
  cudaStream_t get_stream() const { return s_; }
  operator cudaStream_t() const { return s_; }

 private:
  cudaStream_t s_ = nullptr;
};

class launch {
 public:
  explicit launch(const cuda_stream& s) : stream_(s) {}
  const cuda_stream& get_stream() const { return stream_; }

 private:
  const cuda_stream& stream_;
};

namespace exec_tag {
struct timer_t {};
struct sync_t {};
struct no_batch_t {};
inline constexpr timer_t timer{};
inline constexpr sync_t sync{};
inline constexpr no_batch_t no_batch{};
}  // namespace exec_tag

// Event pair a bench brackets its timed region with (exec_tag::timer).
class timer {
 public:
  explicit timer(cudaStream_t s) : s_(s) {
    detail::cuda_check(cudaEventCreate(&e0_), "cudaEventCreate");
    detail::cuda_check(cudaEventCreate(&e1_), "cudaEventCreate");
  }
  ~timer() {
    cudaEventDestroy(e0_);
    cudaEventDestroy(e1_);
  }
  void start() {
    cpu0_ = std::chrono::steady_clock::now();
    detail::cuda_check(cudaEventRecord(e0_, s_), "cudaEventRecord");
    started_ = true;
  }
  void stop() {
    detail::cuda_check(cudaEventRecord(e1_, s_), "cudaEventRecord");
    stopped_ = true;
  }
  // GPU and CPU seconds of the last start/stop pair (synchronises the stop event).
  bool read(double* gpu_s, double* cpu_s) {
    if (!started_ || !stopped_) return false;
    detail::cuda_check(cudaEventSynchronize(e1_), "cudaEventSynchronize");
    *cpu_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - cpu0_).count();
    float ms = 0;
    detail::cuda_check(cudaEventElapsedTime(&ms, e0_, e1_), "cudaEventElapsedTime");
    *gpu_s = ms * 1e-3;
    started_ = stopped_ = false;
    return true;
  }

 private:
  cudaStream_t s_;
  cudaEvent_t e0_ = nullptr, e1_ = nullptr;
  std::chrono::steady_clock::time_point cpu0_;
  bool started_ = false, stopped_ = false;
};

// A named summary value with string attributes (NVBench's summary: "hide",
// "name", "description", ...).
class summary {
 public:
  summary& set_string(const std::string& key, const std::string& v) {
    strings_[key] = v;
    return *this;
  }
  summary& set_float64(const std::string& key, double v) {
    numbers_[key] = v;
    return *this;
  }
  void remove_value(const std::string& key) {
    strings_.erase(key);
    numbers_.erase(key);
  }
  bool has_value(const std::string& key) const { return strings_.count(key) || numbers_.count(key); }
  double get_float64(const std::string& key) const {
    auto it = numbers_.find(key);
    return it == numbers_.end() ? NAN : it->second;
  }
  std::string get_string(const std::string& key) const {
    auto it = strings_.find(key);
    return it == strings_.end() ? std::string() : it->second;
  }

 private:
  std::map<std::string, std::string> strings_;
  std::map<std::string, double> numbers_;
};

struct axis {
  enum kind_t { int64_kind, float64_kind, string_kind } kind;
  std::string name;
  std::vector<int64_t> ints;
  std::vector<double> floats;
  std::vector<std::string> strings;
  size_t size() const { return kind == int64_kind ? ints.size() : kind == float64_kind ? floats.size() : strings.size(); }
  std::string value_text(size_t i) const {
    if (kind == int64_kind) return std::to_string(ints[i]);
    if (kind == float64_kind) {
      std::ostringstream o;
      o << floats[i];
      return o.str();
    }
    return strings[i];
  }
};

struct run_options {
  int min_samples = 10;
  double min_time_s = 0.5;
  double timeout_s = 15.0;
};

class state;
using bench_fn = std::function<void(state&)>;

class benchmark {
 public:
  benchmark(std::string name, bench_fn fn) : name_(std::move(name)), fn_(std::move(fn)) {}
  benchmark& set_name(std::string n) {
    name_ = std::move(n);
    return *this;
  }
  benchmark& add_int64_axis(std::string n, std::vector<int64_t> v) {
    axis a{axis::int64_kind, std::move(n), std::move(v), {}, {}};
    axes_.push_back(std::move(a));
    return *this;
  }
  benchmark& add_float64_axis(std::string n, std::vector<double> v) {
    axis a{axis::float64_kind, std::move(n), {}, std::move(v), {}};
    axes_.push_back(std::move(a));
    return *this;
  }
  benchmark& add_string_axis(std::string n, std::vector<std::string> v) {
    axis a{axis::string_kind, std::move(n), {}, {}, std::move(v)};
    axes_.push_back(std::move(a));
    return *this;
  }
  benchmark& set_min_samples(int n) {
    opts_.min_samples = n;
    return *this;
  }
  benchmark& set_timeout(double s) {
    opts_.timeout_s = s;
    return *this;
  }
  benchmark& set_min_time(double s) {
    opts_.min_time_s = s;
    return *this;
  }
  const std::string& name() const { return name_; }
  std::vector<axis>& axes() { return axes_; }
  const bench_fn& fn() const { return fn_; }
  run_options& options() { return opts_; }

 private:
  std::string name_;
  bench_fn fn_;
  std::vector<axis> axes_;
  run_options opts_;
};

class registry {
 public:
  static registry& get() {
    static registry r;
    return r;
  }
  benchmark& add(const std::string& name, bench_fn fn) {
    benches_.push_back(std::make_unique<benchmark>(name, std::move(fn)));
    return *benches_.back();
  }
  std::vector<std::unique_ptr<benchmark>>& benches() { return benches_; }

 private:
  std::vector<std::unique_ptr<benchmark>> benches_;
};

namespace detail {
// A device buffer written before every sample to evict the L2.
struct l2_flusher {
  void* buf = nullptr;
  size_t bytes = 0;
  void flush(cudaStream_t s) {
    if (!buf) {
      int dev = 0, l2 = 0;
      cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
      cuda_check(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev), "cudaDeviceGetAttribute");
      bytes = std::max<size_t>(2 * (size_t)l2, 1u << 20);
      cuda_check(cudaMalloc(&buf, bytes), "cudaMalloc (L2 flush buffer)");
    }
    cuda_check(cudaMemsetAsync(buf, ++counter & 0xff, bytes, s), "cudaMemsetAsync (L2 flush)");
  }
  int counter = 0;
  static l2_flusher& get() {
    static l2_flusher f;
    return f;
  }
};
}  // namespace detail

class state {
 public:
  state(const benchmark& b, std::map<std::string, std::string> values, const std::vector<axis>& axes,
        run_options opts)
      : bench_(b), values_(std::move(values)), axes_(axes), opts_(opts) {
    for (const char* tag : {"nv/cold/time/gpu/min", "nv/cold/time/gpu/max", "nv/cold/time/cpu/mean",
                            "nv/cold/time/cpu/min", "nv/cold/time/cpu/max", "nv/cold/time/cpu/stdev/relative"})
      summaries_[tag].set_string("hide", "");
  }

  int64_t get_int64(const std::string& name) const { return std::stoll(lookup(name, axis::int64_kind)); }
  double get_float64(const std::string& name) const { return std::stod(lookup(name, axis::float64_kind)); }
  const std::string& get_string(const std::string& name) const { return lookup(name, axis::string_kind); }

  void add_element_count(size_t n, const std::string& column = "") {
    elements_ += n;
    if (!column.empty()) summaries_["nv/element_count/" + column].set_float64("value", (double)n);
  }
  template <typename T>
  void add_global_memory_reads(size_t count, const std::string& = "") {
    gmem_bytes_ += count * sizeof(T);
  }
  template <typename T>
  void add_global_memory_writes(size_t count, const std::string& = "") {
    gmem_bytes_ += count * sizeof(T);
  }
  void skip(const std::string& reason) {
    skipped_ = true;
    skip_reason_ = reason;
  }
  bool is_skipped() const { return skipped_; }
  const std::string& get_skip_reason() const { return skip_reason_; }
  void set_min_samples(int n) { opts_.min_samples = n; }
  void set_timeout(double s) { opts_.timeout_s = s; }
  summary& get_summary(const std::string& tag) { return summaries_[tag]; }
  const std::map<std::string, summary>& get_summaries() const { return summaries_; }
  const cuda_stream& get_cuda_stream() const { return stream_; }
  const std::map<std::string, std::string>& axis_values() const { return values_; }
  const benchmark& get_benchmark() const { return bench_; }

  // Cold measurement of fn(launch&): the whole call is timed.
  template <typename F>
  void exec(F&& fn) {
    measure([&](launch& l, timer& t) {
      t.start();
      fn(l);
      t.stop();
    });
  }
  template <typename F>
  void exec(exec_tag::sync_t, F&& fn) {
    exec(std::forward<F>(fn));
  }
  template <typename F>
  void exec(exec_tag::no_batch_t, F&& fn) {
    exec(std::forward<F>(fn));
  }
  // Cold measurement of the span the bench brackets with timer.start() / stop().
  template <typename F>
  void exec(exec_tag::timer_t, F&& fn) {
    measure(std::forward<F>(fn));
  }

 private:
  const std::string& lookup(const std::string& name, axis::kind_t kind) const {
    for (const axis& a : axes_)
      if (a.name == name && a.kind == kind) return values_.at(name);
    std::fprintf(stderr, "nvbench: benchmark '%s' has no %s axis '%s'\n", bench_.name().c_str(),
                 kind == axis::int64_kind ? "int64" : kind == axis::float64_kind ? "float64" : "string", name.c_str());
    std::exit(2);
  }

  template <typename F>
  void measure(F&& fn) {
    launch l(stream_);
    timer t(stream_);
    std::vector<double> gpu, cpu;
    // one untimed warm-up run (module load, first-touch, lazy set-up)
    fn(l, t);
    detail::cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    double g = 0, c = 0;
    t.read(&g, &c);
    const auto t0 = std::chrono::steady_clock::now();
    double total = 0;
    for (;;) {
      detail::l2_flusher::get().flush(stream_);
      detail::cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
      fn(l, t);
      if (!t.read(&g, &c)) {
        std::fprintf(stderr, "nvbench: %s: exec_tag::timer bench did not call timer.start()/stop()\n",
                     bench_.name().c_str());
        std::exit(2);
      }
      detail::cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
      gpu.push_back(g);
      cpu.push_back(c);
      total += g;
      const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (((int)gpu.size() >= opts_.min_samples && total >= opts_.min_time_s) || wall >= opts_.timeout_s) break;
    }
    record("gpu", gpu);
    record("cpu", cpu);
    summaries_["nv/cold/sample_size"].set_float64("value", (double)gpu.size());
    const double mean = summaries_["nv/cold/time/gpu/mean"].get_float64("value");
    if (elements_) summaries_["nv/element_count"].set_float64("value", elements_ / mean);
    if (gmem_bytes_) summaries_["nv/gmem/bw"].set_float64("value", gmem_bytes_ / mean);
    measured_ = true;
  }

  void record(const char* which, const std::vector<double>& v) {
    const std::string base = std::string("nv/cold/time/") + which + "/";
    double s = 0, mn = INFINITY, mx = 0;
    for (double x : v) {
      s += x;
      mn = std::min(mn, x);
      mx = std::max(mx, x);
    }
    const double mean = s / v.size();
    double var = 0;
    for (double x : v) var += (x - mean) * (x - mean);
    const double sd = v.size() > 1 ? std::sqrt(var / (v.size() - 1)) : 0.0;
    summaries_[base + "mean"].set_float64("value", mean);
    summaries_[base + "min"].set_float64("value", mn);
    summaries_[base + "max"].set_float64("value", mx);
    summaries_[base + "stdev/relative"].set_float64("value", mean > 0 ? sd / mean : 0.0);
  }

  const benchmark& bench_;
  std::map<std::string, std::string> values_;
  const std::vector<axis>& axes_;
  run_options opts_;
  cuda_stream stream_;
  std::map<std::string, summary> summaries_;
  size_t elements_ = 0, gmem_bytes_ = 0;
  bool skipped_ = false, measured_ = false;
  std::string skip_reason_;

 public:
  bool measured() const { return measured_; }
};

namespace detail {

inline std::string fmt_time(double s) {
  char b[64];
  if (!(s == s)) return "-";
  if (s >= 1) std::snprintf(b, sizeof b, "%.3f s", s);
  else if (s >= 1e-3) std::snprintf(b, sizeof b, "%.3f ms", s * 1e3);
  else std::snprintf(b, sizeof b, "%.3f us", s * 1e6);
  return b;
}

// "N=[32,64]", "N=32", "N=[32:128:32]" (int64 range, inclusive), "name=[a,b]" for strings
inline bool parse_axis_override(const std::string& arg, std::string* name, std::vector<std::string>* values,
                                bool* is_range, int64_t range[3]) {
  const size_t eq = arg.find('=');
  if (eq == std::string::npos) return false;
  *name = arg.substr(0, eq);
  std::string v = arg.substr(eq + 1);
  values->clear();
  *is_range = false;
  if (!v.empty() && v.front() == '[' && v.back() == ']') v = v.substr(1, v.size() - 2);
  if (v.find(':') != std::string::npos) {
    int64_t a = 0, b = 0, st = 1;
    char c1 = 0, c2 = 0;
    std::istringstream in(v);
    in >> a >> c1 >> b;
    if (in >> c2 >> st) {}
    if (st <= 0) return false;
    *is_range = true;
    range[0] = a;
    range[1] = b;
    range[2] = st;
    return true;
  }
  std::istringstream in(v);
  std::string item;
  while (std::getline(in, item, ',')) {
    item.erase(0, item.find_first_not_of(' '));
    item.erase(item.find_last_not_of(' ') + 1);
    if (!item.empty()) values->push_back(item);
  }
  return !values->empty();
}

inline void apply_override(benchmark& b, const std::string& arg) {
  std::string name;
  std::vector<std::string> vals;
  bool range = false;
  int64_t r[3];
  if (!parse_axis_override(arg, &name, &vals, &range, r)) {
    std::fprintf(stderr, "nvbench: bad --axis '%s'\n", arg.c_str());
    std::exit(2);
  }
  for (axis& a : b.axes()) {
    if (a.name != name) continue;
    if (a.kind == axis::int64_kind) {
      a.ints.clear();
      if (range)
        for (int64_t x = r[0]; x <= r[1]; x += r[2]) a.ints.push_back(x);
      else
        for (auto& s : vals) a.ints.push_back(std::stoll(s));
    } else if (a.kind == axis::float64_kind) {
      a.floats.clear();
      for (auto& s : vals) a.floats.push_back(std::stod(s));
    } else {
      a.strings = vals;
    }
    return;
  }
  std::fprintf(stderr, "nvbench: benchmark '%s' has no axis '%s'\n", b.name().c_str(), name.c_str());
  std::exit(2);
}

inline std::string csv_escape(const std::string& s) {
  if (s.find_first_of(",\"") == std::string::npos) return s;
  std::string o = "\"";
  for (char c : s) o += (c == '"') ? std::string("\"\"") : std::string(1, c);
  return o + "\"";
}

struct result_row {
  std::string bench;
  std::vector<std::pair<std::string, std::string>> axes;
  std::map<std::string, double> values;
  bool skipped = false;
  std::string skip_reason;
};

inline int run(int argc, char** argv) {
  std::vector<std::string> selected;
  std::vector<std::pair<int, std::string>> overrides;   // (index in `selected` it follows, axis text)
  std::string csv, json;
  int min_samples = -1;
  double timeout = -1, min_time = -1;
  bool list = false;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "nvbench: %s needs a value\n", a.c_str());
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-b" || a == "--benchmark") selected.push_back(next());
    else if (a == "-a" || a == "--axis") overrides.push_back({(int)selected.size() - 1, next()});
    else if (a == "--csv") csv = next();
    else if (a == "--json") json = next();
    else if (a == "--min-samples") min_samples = std::atoi(next().c_str());
    else if (a == "--timeout") timeout = std::atof(next().c_str());
    else if (a == "--min-time") min_time = std::atof(next().c_str());
    else if (a == "-l" || a == "--list") list = true;
    else if (a == "-h" || a == "--help") {
      std::printf(
          "usage: %s [-l] [-b NAME|INDEX]... [-a 'AXIS=[v1,v2]' | -a 'AXIS=[lo:hi:step]']...\n"
          "          [--min-samples N] [--min-time S] [--timeout S] [--csv FILE] [--json FILE]\n"
          "An --axis after a -b applies to that benchmark, before any -b to all of them.\n",
          argv[0]);
      return 0;
    } else {
      std::fprintf(stderr, "nvbench: unknown option %s\n", a.c_str());
      return 2;
    }
  }
  auto& all = registry::get().benches();
  if (list) {
    for (size_t i = 0; i < all.size(); ++i) {
      std::printf("%zu: %s", i, all[i]->name().c_str());
      for (auto& ax : all[i]->axes()) {
        std::printf("  %s=[", ax.name.c_str());
        for (size_t j = 0; j < ax.size(); ++j) std::printf("%s%s", j ? "," : "", ax.value_text(j).c_str());
        std::printf("]");
      }
      std::printf("\n");
    }
    return 0;
  }
  // the benchmarks to run, each with its own copy of the axes
  std::vector<std::pair<benchmark*, std::vector<axis>>> plan;
  auto add_plan = [&](benchmark* b, int sel) {
    std::vector<axis> saved = b->axes();
    for (auto& o : overrides)
      if (o.first == -1 || o.first == sel) apply_override(*b, o.second);
    plan.push_back({b, b->axes()});
    b->axes() = saved;
  };
  if (selected.empty()) {
    for (auto& b : all) add_plan(b.get(), -1);
  } else {
    for (int s = 0; s < (int)selected.size(); ++s) {
      bool found = false;
      for (size_t i = 0; i < all.size(); ++i) {
        if (all[i]->name() == selected[s] || std::to_string(i) == selected[s]) {
          add_plan(all[i].get(), s);
          found = true;
        }
      }
      if (!found) {
        std::fprintf(stderr, "nvbench: no benchmark named '%s'\n", selected[s].c_str());
        return 2;
      }
    }
  }
  int dev = 0;
  cudaDeviceProp prop;
  detail::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  detail::cuda_check(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
  std::vector<result_row> rows;
  for (auto& [b, axes] : plan) {
    run_options opts = b->options();
    if (min_samples > 0) opts.min_samples = min_samples;
    if (timeout > 0) opts.timeout_s = timeout;
    if (min_time >= 0) opts.min_time_s = min_time;
    std::printf("\n# %s\n\n## [%d] %s\n\n", b->name().c_str(), dev, prop.name);
    // header
    std::vector<std::string> shown_tags;
    bool header_done = false;
    size_t combos = 1;
    for (auto& ax : axes) combos *= ax.size();
    for (size_t c = 0; c < combos; ++c) {
      std::map<std::string, std::string> values;
      std::vector<std::pair<std::string, std::string>> ordered;
      size_t rem = c;
      for (auto& ax : axes) {   // first axis varies fastest, as NVBench prints them
        const size_t k = rem % ax.size();
        rem /= ax.size();
        values[ax.name] = ax.value_text(k);
        ordered.push_back({ax.name, ax.value_text(k)});
      }
      state st(*b, values, axes, opts);
      b->fn()(st);
      result_row row{b->name(), ordered, {}, st.is_skipped(), st.get_skip_reason()};
      for (auto& [tag, s] : st.get_summaries())
        if (s.has_value("value")) row.values[tag] = s.get_float64("value");
      if (!header_done) {
        for (auto& [tag, s] : st.get_summaries())
          if (!s.has_value("hide") && s.has_value("value") && tag != "nv/cold/sample_size") shown_tags.push_back(tag);
        std::printf("|");
        for (auto& ax : axes) std::printf(" %s |", ax.name.c_str());
        std::printf(" Samples |");
        for (auto& t : shown_tags) std::printf(" %s |", t.c_str());
        std::printf("\n|");
        for (size_t i = 0; i < axes.size() + 1 + shown_tags.size(); ++i) std::printf("---|");
        std::printf("\n");
        header_done = true;
      }
      std::printf("|");
      for (auto& kv : ordered) std::printf(" %s |", kv.second.c_str());
      if (st.is_skipped()) {
        std::printf(" skipped: %s |\n", st.get_skip_reason().c_str());
      } else {
        std::printf(" %.0f |", row.values["nv/cold/sample_size"]);
        for (auto& t : shown_tags) {
          const double v = row.values.count(t) ? row.values[t] : NAN;
          if (t.rfind("nv/cold/time/", 0) == 0 && t.find("stdev") == std::string::npos)
            std::printf(" %s |", fmt_time(v).c_str());
          else if (t.find("stdev") != std::string::npos)
            std::printf(" %.2f%% |", 100 * v);
          else
            std::printf(" %.4g |", v);
        }
        std::printf("\n");
      }
      std::fflush(stdout);
      rows.push_back(std::move(row));
    }
  }
  if (!csv.empty()) {
    FILE* f = std::fopen(csv.c_str(), "w");
    if (!f) {
      std::fprintf(stderr, "nvbench: cannot write %s\n", csv.c_str());
      return 2;
    }
    std::fprintf(f, "Benchmark,Axes,Skipped,Samples,GPU Time (sec),GPU Noise,GPU Min (sec),GPU Max (sec),"
                    "CPU Time (sec),Elem/s,GlobalMem BW (B/s)\n");
    for (auto& r : rows) {
      std::string ax;
      for (auto& kv : r.axes) ax += (ax.empty() ? "" : " ") + kv.first + "=" + kv.second;
      auto g = [&](const char* t) { return r.values.count(t) ? r.values.at(t) : NAN; };
      std::fprintf(f, "%s,%s,%s,%.0f,%.9g,%.6g,%.9g,%.9g,%.9g,%.6g,%.6g\n", csv_escape(r.bench).c_str(),
                   csv_escape(ax).c_str(), r.skipped ? csv_escape(r.skip_reason).c_str() : "",
                   g("nv/cold/sample_size"), g("nv/cold/time/gpu/mean"), g("nv/cold/time/gpu/stdev/relative"),
                   g("nv/cold/time/gpu/min"), g("nv/cold/time/gpu/max"), g("nv/cold/time/cpu/mean"),
                   g("nv/element_count"), g("nv/gmem/bw"));
    }
    std::fclose(f);
  }
  if (!json.empty()) {
    FILE* f = std::fopen(json.c_str(), "w");
    if (!f) {
      std::fprintf(stderr, "nvbench: cannot write %s\n", json.c_str());
      return 2;
    }
    std::fprintf(f, "{\"device\": \"%s\", \"states\": [", prop.name);
    for (size_t i = 0; i < rows.size(); ++i) {
      const auto& r = rows[i];
      std::fprintf(f, "%s\n {\"benchmark\": \"%s\", \"axes\": {", i ? "," : "", r.bench.c_str());
      for (size_t j = 0; j < r.axes.size(); ++j)
        std::fprintf(f, "%s\"%s\": \"%s\"", j ? ", " : "", r.axes[j].first.c_str(), r.axes[j].second.c_str());
      std::fprintf(f, "}, \"skipped\": %s, \"summaries\": {", r.skipped ? "true" : "false");
      size_t j = 0;
      for (auto& [tag, v] : r.values)
        if (v == v) std::fprintf(f, "%s\"%s\": %.9g", j++ ? ", " : "", tag.c_str(), v);
      std::fprintf(f, "}}");
    }
    std::fprintf(f, "\n]}\n");
    std::fclose(f);
  }
  return 0;
}
}  // namespace detail

}  // namespace nvbench

#define NVBENCH_COMPAT_CAT2(a, b) a##b
#define NVBENCH_COMPAT_CAT(a, b) NVBENCH_COMPAT_CAT2(a, b)
// Registers `fn` (void fn(nvbench::state&)) at static-initialisation time and
// returns its benchmark for the chained set_name / add_*_axis calls.
#define NVBENCH_BENCH(fn)                                                            \
  static ::nvbench::benchmark& NVBENCH_COMPAT_CAT(nvbench_compat_bench_, __LINE__) = \
      ::nvbench::registry::get().add(#fn, fn)
#define NVBENCH_MAIN \
  int main(int argc, char** argv) { return ::nvbench::detail::run(argc, argv); }
