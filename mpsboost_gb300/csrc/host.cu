// Host side of the CUDA backend: the C ABI of include/mpsb_cuda.h, the device-resident
// dataset, the node-level entries of the reference backend contract
// (include/mpsboost/backend.hpp:52-135) and the device-resident training session.
//
// One backend owns one CUDA stream. A training session keeps every input on the device
// and runs each boosting round as a fixed sequence of kernels (gradients, then per depth
// level: zero slots, histogram build, root stats or sibling subtraction, split scan,
// finalize, partition; then leaf application), captured once as a CUDA graph and
// replayed per round. No row ever returns to the host inside a round; the host reads
// back only the finished trees.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "host_types.h"

using namespace mpsb;

namespace mpsb {

thread_local std::string g_error;

// MPSB_TRACE=1: host-side phase times of session setup and export on stderr.
struct PhaseTrace {
  bool on = false;
  std::chrono::steady_clock::time_point t0, last;
  const char* what;
  explicit PhaseTrace(const char* w) : what(w) {
    const char* v = std::getenv("MPSB_TRACE");
    on = v && std::atoi(v) != 0;
    t0 = last = std::chrono::steady_clock::now();
  }
  void mark(const char* phase) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[mpsb %s] %-28s %8.3f ms (total %8.3f)\n", what, phase,
                 std::chrono::duration<double, std::milli>(now - last).count(),
                 std::chrono::duration<double, std::milli>(now - t0).count());
    last = now;
  }
};

std::string describe_device_error(uint32_t bits) {
  std::string m = "device reported:";
  if (bits & kErrCountMismatch) m += " Histogram sample count does not match node statistics;";
  if (bits & kErrNonFinite) m += " non-finite histogram, gain or leaf value;";
  if (bits & kErrHessian) m += " Histogram G/H must be finite and Hessian non-negative;";
  if (bits & kErrSubtraction) m += " Histogram subtraction child exceeded parent;";
  if (bits & kErrPartition) m += " Sample partition counts do not match histogram statistics;";
  if (bits & kErrMissing) m += " missing statistics exceed parent statistics;";
  if (bits & kErrCapacity) m += " internal capacity exceeded;";
  if (bits & kErrGradient) m += " invalid label, prediction, weight or gradient;";
  if (bits & kErrPrefix) m += " non-missing histogram prefix exceeded parent;";
  if (bits & kErrRootCache) m += " hessian scale of the reused root histogram changed;";
  if (bits & kErrLeafQueue) m += " leaf-wise active queue reached max_active_leaves;";
  if (bits & kErrCopy) m += " a tensor copy of the histogram build did not complete;";
  return m;
}

// MPSB_HIST_TMA=1: row-major histogram levels stage their gathered rows with TMA gather4
// copies through this map instead of cp.async. Off by default: on GB300 the gather4 path
// builds the depth-8 levels about 8 % slower than cp.async (the copies complete later and
// the warps wait on them), although it takes the row loads off the L1 tag stage.
void attach_bins_tmap(mpsb_cuda_dataset* d) {
  d->has_bins_tmap = false;
  const char* v = std::getenv("MPSB_HIST_TMA");
  if (!v || std::atoi(v) == 0 || d->slots != uint32_t(kSlots)) return;
  d->has_bins_tmap = encode_bins_tmap(&d->bins_tmap, d->bins.as<uint8_t>(),
                                      uint64_t(d->nfb) * kBlockFeatures, d->n_rows);
}

uint32_t dataset_slots(const uint32_t* bin_count, const uint8_t* has_missing, uint32_t features) {
  uint64_t need = 0;
  for (uint32_t f = 0; f < features; ++f) {
    if (bin_count[f] == 0) throw DataError("every feature needs at least one bin");
    if (bin_count[f] > 65536) throw DataError("a feature may have at most 65536 bins");
    const uint64_t n = uint64_t(bin_count[f]) + (has_missing && has_missing[f] ? 1 : 0);
    if (n > 65536)
      throw UnsupportedError("a feature with missing values may have at most 65535 bins on the CUDA backend");
    need = std::max(need, n);
  }
  if (need <= uint64_t(kSlots)) return uint32_t(kSlots);
  return uint32_t((need + kSlots - 1) / kSlots * kSlots);
}

// ---- reference semantics evaluated on the host --------------------------------------
void validate_tree_params(const mpsb_train_params& p, uint32_t features) {  // tree_structure.cpp:17-52
  if (p.min_samples_leaf == 0) throw TrainingError("min_samples_leaf must be at least 1");
  if (p.max_leaves == 1) throw TrainingError("max_leaves must be zero or at least 2");
  if (p.max_active_leaves == 1) throw TrainingError("max_active_leaves must be zero or at least 2");
  if (p.max_active_leaves != 0 && p.max_leaves != 0 && p.max_active_leaves > p.max_leaves)
    throw TrainingError("max_active_leaves must not exceed max_leaves");
  auto nonneg = [](double v, const char* what) {
    if (!std::isfinite(v) || v < 0.0) throw TrainingError(std::string(what) + " must be finite and non-negative");
  };
  nonneg(p.min_child_weight, "min_child_weight");
  nonneg(p.reg_lambda, "reg_lambda");
  nonneg(p.reg_alpha, "reg_alpha");
  nonneg(p.max_delta_step, "max_delta_step");
  nonneg(p.gamma, "gamma");
  nonneg(p.min_gain_to_split, "min_gain_to_split");
  if (p.n_monotonic != 0 && p.n_monotonic != features)
    throw TrainingError("monotonic_constraints length must match feature count");
  for (uint32_t i = 0; i < p.n_monotonic; ++i)
    if (p.monotonic_constraints[i] < -1 || p.monotonic_constraints[i] > 1)
      throw TrainingError("monotonic_constraints values must be -1, 0, or 1");
  for (uint32_t g = 0; g < p.n_interaction_groups; ++g) {  // tree_interactions.cpp:57-70
    if (p.interaction_offsets[g + 1] == p.interaction_offsets[g])
      throw TrainingError("interaction constraint groups must be non-empty");
    for (uint32_t i = p.interaction_offsets[g]; i < p.interaction_offsets[g + 1]; ++i)
      if (p.interaction_features[i] >= features)
        throw TrainingError("interaction constraint feature index out of range");
  }
  if (p.split_strategy > 1) throw TrainingError("unknown split strategy");
  if (p.growth_strategy > 1) throw TrainingError("unknown growth strategy");
}

void validate_training_params(const mpsb_train_params& p) {  // trainer.cpp:22-42
  if (p.n_estimators == 0) throw TrainingError("n_estimators must be at least 1");
  if (!std::isfinite(p.learning_rate) || p.learning_rate <= 0.0 || p.learning_rate > 1.0)
    throw TrainingError("learning_rate must be in (0, 1]");
  if (p.max_bins < 2 || p.max_bins > 65536) throw TrainingError("max_bins must be in [2, 65536]");
  if (!std::isfinite(p.objective_alpha) || p.objective_alpha <= 0.0 || p.objective_alpha >= 1.0)
    throw TrainingError("quantile alpha must be in (0, 1)");
  if (!std::isfinite(p.tweedie_variance_power) || p.tweedie_variance_power <= 1.0 ||
      p.tweedie_variance_power >= 2.0)
    throw TrainingError("tweedie variance power must be in (1, 2)");
  if (p.objective > 4) throw TrainingError("unknown training objective");
}

// One pass over the rows: the weight total of ValidateWeights (trainer.cpp:44-66) and,
// for the mean-type objectives (label_mode 1: squared error, finite labels; 2: poisson and
// tweedie, non-negative labels), the weighted label sum of InitialBaseScore
// (trainer.cpp:68-176), both accumulated in row order as the reference does. The two sums
// are independent chains, so one loop costs about one chain. Errors keep the reference's
// order: every weight check before any label check, each at its first failing row.
struct RowSums {
  double total = 0.0;      // sum of weights
  double label_sum = 0.0;  // sum of label * weight (label_mode != 0)
  int label_mode = 0;
};

// The reference's sequential loop, which also finds the first failing row and its error.
RowSums row_sums_checked(const double* w, const double* y, uint64_t n, int label_mode,
                         const char* name) {
  RowSums r;
  r.label_mode = y ? label_mode : 0;
  double total = 0.0, s = 0.0;
  uint64_t w_bad = n, w_ovf = n, y_bad = n, y_ovf = n;
  for (uint64_t i = 0; i < n; ++i) {
    const double x = w ? w[i] : 1.0;
    if (!std::isfinite(x) || x < 0.0) { w_bad = i; break; }
    total += x;
    if (!std::isfinite(total)) { w_ovf = i; break; }
    if (r.label_mode && y_bad == n && y_ovf == n) {
      const double v = y[i];
      if (!std::isfinite(v) || (r.label_mode == 2 && v < 0.0)) {
        y_bad = i;
      } else {
        s += v * x;
        if (!std::isfinite(s)) y_ovf = i;
      }
    }
  }
  if (w_bad < n) throw TrainingError("sample weights must be finite non-negative values");
  if (w_ovf < n) throw TrainingError("sample weight sum overflowed");
  if (total <= 0.0) throw TrainingError("sample weights must contain positive total weight");
  if (y_bad < n) {
    if (r.label_mode == 1) throw TrainingError("Labels must be finite");
    throw TrainingError(std::string(name) + " labels must be non-negative");
  }
  if (y_ovf < n) {
    if (r.label_mode == 1) throw TrainingError("Label accumulation overflowed");
    throw TrainingError(std::string(name) + " label sum overflowed");
  }
  r.total = total;
  r.label_sum = s;
  return r;
}

// Fast path: the two row-order sums in a tight loop (the same additions, so the same
// results) while worker threads check every weight and label; any failed check or
// non-finite sum reruns the sequential loop above for the reference's exact error.
RowSums row_sums(const double* w, const double* y, uint64_t n, int label_mode, const char* name) {
  if (n == 0) throw TrainingError("labels must be non-empty");
  const int mode = y ? label_mode : 0;
  std::atomic<bool> bad{false};
  const uint32_t workers = uint32_t(std::min<uint64_t>(
      std::max(1u, std::min(16u, std::thread::hardware_concurrency())), (n + (1u << 20) - 1) >> 20));
  auto check = [&](uint32_t k, uint32_t of) {
    const uint64_t lo = n * k / of, hi = n * (k + 1) / of;
    bool ok = true;
    for (uint64_t i = lo; i < hi; ++i) {
      const double x = w ? w[i] : 1.0;
      ok &= std::isfinite(x) && !(x < 0.0);
      if (mode) {
        const double v = y[i];
        ok &= std::isfinite(v) && !(mode == 2 && v < 0.0);
      }
    }
    if (!ok) bad.store(true, std::memory_order_relaxed);
  };
  std::vector<std::thread> pool;
  if (workers > 1)
    for (uint32_t k = 0; k < workers; ++k) pool.emplace_back(check, k, workers);
  else
    check(0, 1);
  double total = 0.0, s = 0.0;
  if (mode) {
    for (uint64_t i = 0; i < n; ++i) {
      const double x = w ? w[i] : 1.0;
      total += x;
      s += y[i] * x;
    }
  } else if (w) {
    for (uint64_t i = 0; i < n; ++i) total += w[i];
  } else {
    for (uint64_t i = 0; i < n; ++i) total += 1.0;
  }
  for (auto& t : pool) t.join();
  if (bad.load() || !std::isfinite(total) || !(total > 0.0) || (mode && !std::isfinite(s)))
    return row_sums_checked(w, y, n, label_mode, name);
  RowSums r;
  r.label_mode = mode;
  r.total = total;
  r.label_sum = s;
  return r;
}

double validate_weights(const double* w, uint64_t n) {  // trainer.cpp:44-66
  return row_sums(w, nullptr, n, 0, nullptr).total;
}

const char* count_objective_name(uint32_t objective) {
  return objective == MPSB_POISSON ? "poisson" : "tweedie";
}

// The label mode of row_sums for a boosting objective (0: the base score needs another pass).
int label_mode_of(uint32_t objective) {
  if (objective == MPSB_SQUARED_ERROR) return 1;
  if (objective == MPSB_POISSON || objective == MPSB_TWEEDIE) return 2;
  return 0;
}

// InitialBaseScore (trainer.cpp:68-176) on host FP64 in row order. `cls` >= 0 selects the
// one-vs-rest binary labels (label == cls). `pre`: this fit's row sums, when they carry
// the label sum of the objective (cls < 0).
double base_score(const mpsb_train_params& p, const double* y, const double* w, uint64_t n,
                  int64_t cls, const RowSums* pre = nullptr) {
  const int mode = cls < 0 ? label_mode_of(p.objective) : 0;
  if (mode && pre && pre->label_mode == mode) {
    if (mode == 1) return pre->label_sum / pre->total;
    return std::log(std::max(1e-15, pre->label_sum / pre->total));
  }
  if (mode) {
    const RowSums r = row_sums(w, y, n, mode, count_objective_name(p.objective));
    if (mode == 1) return r.label_sum / r.total;
    return std::log(std::max(1e-15, r.label_sum / r.total));
  }
  const double total = pre ? pre->total : validate_weights(w, n);
  auto W = [&](uint64_t i) { return w ? w[i] : 1.0; };
  auto Y = [&](uint64_t i) { return cls >= 0 ? (y[i] == double(cls) ? 1.0 : 0.0) : y[i]; };
  switch (p.objective) {
    case MPSB_BINARY_LOGISTIC: {
      double pos = 0.0;
      for (uint64_t i = 0; i < n; ++i) {
        const double l = Y(i);
        if (l == 0.0) continue;
        if (l == 1.0) { pos += W(i); continue; }
        throw TrainingError("binary-logistic labels must be 0 or 1");
      }
      const double eps = 1e-15;
      double prob = pos / total;
      prob = std::min(1.0 - eps, std::max(eps, prob));
      return std::log(prob / (1.0 - prob));
    }
    case MPSB_QUANTILE: {
      std::vector<std::pair<double, double>> o(n);
      for (uint64_t i = 0; i < n; ++i) {
        if (!std::isfinite(Y(i))) throw TrainingError("label must be finite");
        o[i] = {Y(i), W(i)};
      }
      std::sort(o.begin(), o.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
      const double thr = p.objective_alpha * total;
      double cum = 0.0;
      for (const auto& it : o) {
        cum += it.second;
        if (cum >= thr) return it.first;
      }
      return o.back().first;
    }
    default:  // squared error, poisson and tweedie take the row_sums path above
      throw TrainingError("unknown training objective");
  }
}

// Runs body(0..count-1) on worker threads (each index once); rethrows the first error.
template <class F>
void parallel_trees(uint32_t count, F&& body) {
  const uint32_t workers = std::min<uint32_t>(count, std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<uint32_t> next{0};
  std::vector<std::exception_ptr> errors(workers);
  auto run = [&](uint32_t w) {
    try {
      for (uint32_t i = next.fetch_add(1); i < count; i = next.fetch_add(1)) body(i);
    } catch (...) {
      errors[w] = std::current_exception();
    }
  };
  std::vector<std::thread> pool;
  for (uint32_t w = 1; w < workers; ++w) pool.emplace_back(run, w);
  if (workers > 0) run(0);
  for (auto& t : pool) t.join();
  for (auto& e : errors)
    if (e) std::rethrow_exception(e);
}

// InitialBaseScore of a mean-type objective (label_mode 1 or 2) over a row multiset in
// row order, row r taken m[r] times: the same sequence of additions as over the expanded
// sample, without expanding it.
double multiset_base_score(const mpsb_train_params& p, const double* y, const double* w,
                           const uint8_t* m, uint64_t n, int mode) {
  double total = 0.0, s = 0.0;
  bool bad_w = false, bad_y = false;
  for (uint64_t r = 0; r < n; ++r) {
    for (uint32_t c = 0; c < m[r]; ++c) {
      const double x = w ? w[r] : 1.0;
      total += x;
      s += y[r] * x;
    }
    if (m[r]) {
      const double x = w ? w[r] : 1.0;
      bad_w |= !std::isfinite(x) || x < 0.0;
      bad_y |= !std::isfinite(y[r]) || (mode == 2 && y[r] < 0.0);
    }
  }
  if (bad_w || bad_y || !std::isfinite(total) || !(total > 0.0) || !std::isfinite(s)) {
    // The exact error of the reference's sequential checks, over the expanded sample.
    std::vector<double> ys, ws;
    for (uint64_t r = 0; r < n; ++r)
      for (uint32_t c = 0; c < m[r]; ++c) {
        ys.push_back(y[r]);
        if (w) ws.push_back(w[r]);
      }
    return base_score(p, ys.data(), w ? ws.data() : nullptr, ys.size(), -1);
  }
  if (mode == 1) return s / total;
  return std::log(std::max(1e-15, s / total));
}

uint32_t effective_max_leaves(const mpsb_train_params& p) {  // tree_structure.cpp:54-62
  if (p.max_leaves != 0) return p.max_leaves;
  if (p.max_depth >= 31) return 0xFFFFFFFFu;
  return 1u << p.max_depth;
}

// Fixed-point exponents of one set of FP32 pairs (same rule as the round_setup kernel).
void fixed_scales(const float* pairs32, uint64_t n, uint64_t n_rows, int32_t* kg, int32_t* kh) {
  float mg = 0.0f, mh = 0.0f;
  for (uint64_t i = 0; i < n; ++i) {
    mg = std::max(mg, std::fabs(pairs32[2 * i]));
    mh = std::max(mh, std::max(pairs32[2 * i + 1], 0.0f));
  }
  (void)n_rows;
  int e;
  std::frexp(mg, &e);
  *kg = mg > 0.0f ? 30 - e : 0;
  std::frexp(mh, &e);
  *kh = mh > 0.0f ? 30 - e : 0;
}

}  // namespace mpsb

// ======================================================================================
// Backend
// ======================================================================================
extern "C" {

const char* mpsb_cuda_last_error(void) { return g_error.c_str(); }
int mpsb_cuda_abi_version(void) { return MPSB_CUDA_ABI_VERSION; }

int mpsb_cuda_device_count(int* out) {
  return guard([&] {
    if (out == nullptr) throw TrainingError("output pointer must not be null");
    *out = 0;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {  // no driver or no device
      cudaGetLastError();
      return;
    }
    int usable = 0;
    for (int d = 0; d < count; ++d) {
      int major = 0, minor = 0;
      if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, d) == cudaSuccess &&
          cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, d) == cudaSuccess &&
          major == 10 && minor == 3)
        ++usable;
    }
    cudaGetLastError();
    *out = usable;
  });
}

int mpsb_cuda_backend_create(int device, mpsb_cuda_backend** out) {
  return guard([&] {
    if (out == nullptr) throw TrainingError("output pointer must not be null");
    int count = 0;
    CK(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) throw BackendError("CUDA device index out of range");
    std::unique_ptr<mpsb_cuda_backend> b(new mpsb_cuda_backend);
    b->device = device;
    CK(cudaSetDevice(device));
    CK(cudaGetDeviceProperties(&b->prop, device));
    if (b->prop.major != 10 || b->prop.minor != 3)
      throw BackendError("the CUDA backend is built for sm_103a (GB300); device " +
                         std::string(b->prop.name) + " has compute capability " +
                         std::to_string(b->prop.major) + "." + std::to_string(b->prop.minor));
    b->sm_count = b->prop.multiProcessorCount;
    CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&b->t0));
    CK(cudaEventCreate(&b->t1));
    b->error.alloc(sizeof(uint32_t));
    CK(cudaMemset(b->error.p, 0, sizeof(uint32_t)));
    *out = b.release();
  });
}

void mpsb_cuda_backend_destroy(mpsb_cuda_backend* b) { delete b; }

int mpsb_cuda_backend_info(const mpsb_cuda_backend* b, mpsb_cuda_info* out) {
  return guard([&] {
    std::memset(out, 0, sizeof *out);
    out->available = 1;
    out->sm_count = uint32_t(b->sm_count);
    out->cc_major = uint32_t(b->prop.major);
    out->cc_minor = uint32_t(b->prop.minor);
    out->total_memory = b->prop.totalGlobalMem;
    std::snprintf(out->device_name, sizeof out->device_name, "%.95s", b->prop.name);
  });
}

int mpsb_cuda_backend_set_hist_mode(mpsb_cuda_backend* b, int mode) {
  return guard([&] {
    if (mode != MPSB_HIST_FIXED && mode != MPSB_HIST_FLOAT) throw TrainingError("unknown histogram mode");
    b->hist_mode = mode;
  });
}

int mpsb_cuda_timer_begin(mpsb_cuda_backend* b) {
  return guard([&] { CK(cudaEventRecord(b->t0, b->stream)); });
}

int mpsb_cuda_timer_end(mpsb_cuda_backend* b, float* ms) {
  return guard([&] {
    CK(cudaEventRecord(b->t1, b->stream));
    CK(cudaEventSynchronize(b->t1));
    CK(cudaEventElapsedTime(ms, b->t0, b->t1));
  });
}

int mpsb_cuda_synchronize(mpsb_cuda_backend* b) {
  return guard([&] { CK(cudaStreamSynchronize(b->stream)); });
}

int mpsb_cuda_host_register(void* p, uint64_t bytes) {
  return guard([&] { CK(cudaHostRegister(p, bytes, cudaHostRegisterDefault)); });
}

int mpsb_cuda_host_unregister(void* p) {
  return guard([&] { CK(cudaHostUnregister(p)); });
}

// ---- binning ---------------------------------------------------------------------------
int mpsb_quantize_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                        uint64_t rs, uint64_t cs, uint32_t max_bins, uint32_t n_threads,
                        void* bins, uint8_t* missing, float* boundaries,
                        uint64_t* boundary_offset, uint32_t* boundary_count,
                        uint32_t* bin_count, uint64_t* missing_count) {
  return guard([&] {
    mpsb::quantize_dense(data, scalar_type, rows, features, rs, cs, max_bins, n_threads, bins,
                         missing, boundaries, boundary_offset, boundary_count, bin_count,
                         missing_count);
  });
}

int mpsb_transform_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                         uint64_t rs, uint64_t cs, uint32_t max_bins, const float* boundaries,
                         const uint64_t* boundary_offset, const uint32_t* boundary_count,
                         uint32_t n_threads, void* bins, uint8_t* missing) {
  return guard([&] {
    mpsb::transform_dense(data, scalar_type, rows, features, rs, cs, max_bins, boundaries,
                          boundary_offset, boundary_count, n_threads, bins, missing);
  });
}

}  // extern "C"

// ---- dataset ---------------------------------------------------------------------------
namespace mpsb {

void dataset_ready(const mpsb_cuda_dataset* d) {
  if (d == nullptr) return;
  std::lock_guard<std::mutex> lock(d->ready_mutex);
  if (d->pending) {
    d->backend->activate();
    CK(cudaEventSynchronize(d->ready));
    uint32_t e = 0;
    CK(cudaMemcpy(&e, d->pack_error.p, sizeof e, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 2; ++k) {
      d->stage[k].reset();
      d->mstage[k].reset();
    }
    d->pending = false;
    d->invalid = e != 0;
  }
  if (d->invalid) throw DataError("Binned value exceeds the feature histogram range");
}

namespace {

// Allocates the dataset and enqueues its upload and pack; returns before they complete
// (the dataset is pending).
std::unique_ptr<mpsb_cuda_dataset> start_dataset(mpsb_cuda_backend* b, const void* bins,
                                                 uint32_t width, const uint8_t* missing,
                                                 uint64_t rows, uint32_t features,
                                                 const uint32_t* bin_count) {
  if (!b || !bins || !bin_count) throw TrainingError("null argument");
  if (width != 1 && width != 2) throw DataError("bin width must be 1 or 2 bytes");
  if (rows == 0 || features == 0) throw DataError("dataset must contain at least one row and one feature");
  if (rows >= 0xFFFFFFFFull) throw UnsupportedError("the CUDA backend indexes rows with uint32");
  b->activate();
  PhaseTrace trace("dataset");
  std::unique_ptr<mpsb_cuda_dataset> d(new mpsb_cuda_dataset);
  d->backend = b;
  d->n_rows = uint32_t(rows);
  d->features = features;
  d->nfb = (features + kBlockFeatures - 1) / kBlockFeatures;
  d->h_bin_count.assign(bin_count, bin_count + features);
  d->h_has_missing.assign(features, 0);
  if (missing) {
    for (uint32_t f = 0; f < features; ++f) {
      const uint8_t* m = missing + uint64_t(f) * rows;
      for (uint64_t r = 0; r < rows; ++r)
        if (m[r]) { d->h_has_missing[f] = 1; break; }
    }
  }
  d->slots = dataset_slots(bin_count, d->h_has_missing.data(), features);
  const bool wide = d->slots != uint32_t(kSlots);
  trace.mark("bin counts, missing scan");
  d->bin_count.alloc(features * sizeof(uint32_t));
  d->has_missing.alloc(features);
  CK(cudaMemcpyAsync(d->bin_count.p, bin_count, features * sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(d->has_missing.p, d->h_has_missing.data(), features, cudaMemcpyHostToDevice, b->stream));
  if (wide) {
    d->bins16.alloc(size_t(d->nfb) * rows * kBlockFeatures * sizeof(uint16_t));
    d->bins16_fm.alloc(size_t(features) * rows * sizeof(uint16_t));
  } else {
    d->bins.alloc(size_t(d->nfb) * rows * kBlockFeatures);
    d->bins_blocked.alloc(size_t(d->nfb) * rows * kBlockFeatures);
    d->bins_fm.alloc(size_t(features) * rows);
  }
  d->pack_error.alloc(sizeof(uint32_t));
  CK(cudaMemsetAsync(d->pack_error.p, 0, sizeof(uint32_t), b->stream));
  CK(cudaEventCreateWithFlags(&d->ready, cudaEventDisableTiming));
  trace.mark("allocs");
  // Feature block by feature block (32 feature columns, contiguous in the feature-major
  // source): the copy stream uploads block fb + 1 into one staging buffer while the
  // compute stream packs block fb from the other.
  if (!b->copy_stream) CK(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
  const size_t block_cells = size_t(kBlockFeatures) * rows;
  DevBuf* stage = d->stage;
  DevBuf* mstage = d->mstage;
  const int nstage = d->nfb > 1 ? 2 : 1;
  for (int k = 0; k < nstage; ++k) {
    stage[k].alloc(block_cells * width);
    if (missing) mstage[k].alloc(block_cells);
  }
  struct Events {
    cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
    ~Events() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } ev;  // copied[2], packed[2]
  for (cudaEvent_t& x : ev.e) CK(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
  for (uint32_t fb = 0; fb < d->nfb; ++fb) {
    const int k = int(fb & 1);
    const uint32_t nf = std::min<uint32_t>(kBlockFeatures, features - fb * kBlockFeatures);
    const size_t first = size_t(fb) * block_cells;
    if (fb >= 2) CK(cudaStreamWaitEvent(b->copy_stream, ev.e[2 + k], 0));  // block fb-2 packed
    CK(cudaMemcpyAsync(stage[k].p, static_cast<const uint8_t*>(bins) + first * width,
                       size_t(nf) * rows * width, cudaMemcpyHostToDevice, b->copy_stream));
    if (missing)
      CK(cudaMemcpyAsync(mstage[k].p, missing + first, size_t(nf) * rows, cudaMemcpyHostToDevice,
                         b->copy_stream));
    CK(cudaEventRecord(ev.e[k], b->copy_stream));
    CK(cudaStreamWaitEvent(b->stream, ev.e[k], 0));
    if (wide)
      CK(launch_pack_bins16_block(stage[k].p, width, missing ? mstage[k].as<uint8_t>() : nullptr,
                                  d->bin_count.as<uint32_t>(), d->n_rows, features, fb, d->slots,
                                  d->bins16.as<uint16_t>(), d->bins16_fm.as<uint16_t>(),
                                  d->pack_error.as<uint32_t>(), b->stream));
    else
      CK(launch_pack_bins_block(stage[k].p, width, missing ? mstage[k].as<uint8_t>() : nullptr,
                                d->bin_count.as<uint32_t>(), d->n_rows, features, d->nfb, fb,
                                d->bins.as<uint8_t>(), d->bins_blocked.as<uint8_t>(),
                                d->bins_fm.as<uint8_t>(), d->pack_error.as<uint32_t>(), b->stream));
    CK(cudaEventRecord(ev.e[2 + k], b->stream));
  }
  CK(cudaEventRecord(d->ready, b->stream));
  d->pending = true;
  trace.mark("upload + pack (enqueued)");
  attach_bins_tmap(d.get());
  return d;
}

}  // namespace
}  // namespace mpsb

extern "C" {

int mpsb_cuda_dataset_create(mpsb_cuda_backend* b, const void* bins, uint32_t width,
                             const uint8_t* missing, uint64_t rows, uint32_t features,
                             const uint32_t* bin_count, mpsb_cuda_dataset** out) {
  return guard([&] {
    if (!out) throw TrainingError("null argument");
    std::unique_ptr<mpsb_cuda_dataset> d = start_dataset(b, bins, width, missing, rows, features, bin_count);
    PhaseTrace trace("dataset");
    dataset_ready(d.get());
    trace.mark("upload + pack (synchronized)");
    *out = d.release();
  });
}

int mpsb_cuda_dataset_create_async(mpsb_cuda_backend* b, const void* bins, uint32_t width,
                                   const uint8_t* missing, uint64_t rows, uint32_t features,
                                   const uint32_t* bin_count, mpsb_cuda_dataset** out) {
  return guard([&] {
    if (!out) throw TrainingError("null argument");
    *out = start_dataset(b, bins, width, missing, rows, features, bin_count).release();
  });
}

int mpsb_cuda_dataset_wait(const mpsb_cuda_dataset* d) {
  return guard([&] {
    if (!d) throw TrainingError("null argument");
    dataset_ready(d);
  });
}

void mpsb_cuda_dataset_destroy(mpsb_cuda_dataset* d) { delete d; }

int mpsb_cuda_dataset_uses_tma(const mpsb_cuda_dataset* d) { return d && d->has_bins_tmap ? 1 : 0; }

}  // extern "C"

// ======================================================================================
// Autotuned launch shapes, per fit shape
// ======================================================================================
namespace mpsb {

struct TuneKey {
  uint32_t rows, features, depth, mode, unit_hess, weighted, leafwise;
  bool operator<(const TuneKey& o) const {
    return std::tie(rows, features, depth, mode, unit_hess, weighted, leafwise) <
           std::tie(o.rows, o.features, o.depth, o.mode, o.unit_hess, o.weighted, o.leafwise);
  }
};

std::mutex g_tune_mutex;
std::map<TuneKey, mpsb_cuda_tuning> g_tune_table;

// The shape of a single-model fit (forests, softmax and one-vs-rest keep the built-in
// launch shape).
bool unit_hessian_fit(const double* weights, const mpsb_train_params& p) {
  bool unit = !weights && (p.objective == MPSB_SQUARED_ERROR || p.objective == MPSB_QUANTILE);
  if (const char* v = std::getenv("MPSB_UNIT_HESS")) unit = unit && std::atoi(v) != 0;
  return unit;
}

TuneKey tune_key_of(const mpsb_cuda_dataset* ds, const double* weights, const mpsb_train_params& p,
                    uint32_t options) {
  return TuneKey{ds->n_rows, ds->features, p.max_depth,
                 uint32_t((options & MPSB_OPT_FLOAT_HIST) ? kModeFloat : kModeFixed),
                 unit_hessian_fit(weights, p) ? 1u : 0u, weights ? 1u : 0u,
                 p.growth_strategy == 1 ? 1u : 0u};
}

bool tuned_shape(const TuneKey& k, mpsb_cuda_tuning* out) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  const auto it = g_tune_table.find(k);
  if (it == g_tune_table.end()) return false;
  *out = it->second;
  return true;
}

}  // namespace mpsb

// ======================================================================================
// Training session
// ======================================================================================
struct mpsb_cuda_trainer {
  mpsb_cuda_backend* b = nullptr;
  const mpsb_cuda_dataset* ds = nullptr;
  mpsb_train_params params{};
  uint32_t options = 0;
  uint32_t depth = 0;
  uint32_t n_trees = 1;
  bool ovr = false;
  TrainerDev dev{};
  HistConfig hcfg;
  std::vector<std::unique_ptr<DevBuf>> bufs;
  std::vector<double> base_scores;
  // One graph for a full round and one for a round that reuses the roots' count and
  // hessian histograms.
  cudaGraph_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
  bool leafwise = false;   // growth_strategy leaf_wise: steps instead of depth levels
  uint32_t lw_steps = 0;    // split steps per tree and round (max leaves - 1)
  bool root_reuse = false;  // the hessian does not depend on the prediction
  uint32_t softmax_classes = 0;  // native softmax: one tree per class per round
  bool root_saved = false;  // a round has saved the roots' count/hessian histograms
  std::vector<cudaEvent_t> events;  // 2 per level (histogram build begin/end)
  unsigned long long* level_cells = nullptr;  // device: ctl->cells after each level's build
  std::vector<double> level_ms;
  std::vector<uint64_t> level_cells_total;
  uint32_t rounds_enqueued = 0;
  uint32_t blocked_levels = 2;  // levels built from the column-blocked bins
  mpsb_cuda_stats stats{};
  uint64_t kernels_per_round[2] = {0, 0};
  uint64_t cells_base = 0, rows_base = 0, part_base = 0;
  unsigned long long cells_before_round = 0;

  template <class T>
  T* alloc(size_t count) {
    bufs.emplace_back(new DevBuf);
    bufs.back()->alloc(count * sizeof(T));
    return bufs.back()->as<T>();
  }

  cudaStream_t side = nullptr;                      // work beside the main stream
  cudaEvent_t fork_ev = nullptr, zero_ev = nullptr;  // fork to / join from `side`

  ~mpsb_cuda_trainer() {
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (zero_ev) cudaEventDestroy(zero_ev);
    if (side) cudaStreamDestroy(side);
    for (int i = 0; i < 2; ++i) {
      if (graph_exec[i]) cudaGraphExecDestroy(graph_exec[i]);
      if (graph[i]) cudaGraphDestroy(graph[i]);
    }
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  }

  int grid(int per_sm) const { return b->sm_count * per_sm; }

  // Captured rounds bake in the launch shape: drop them after a change.
  void reset_graphs() {
    for (int i = 0; i < 2; ++i) {
      if (graph_exec[i]) cudaGraphExecDestroy(graph_exec[i]);
      if (graph[i]) cudaGraphDestroy(graph[i]);
      graph_exec[i] = nullptr;
      graph[i] = nullptr;
    }
  }

  void apply_shape(const mpsb_cuda_tuning& s) {
    hcfg.threads = int(s.hist_threads);
    hcfg.stages = int(s.hist_stages);
    hcfg.root_threads = int(s.root_threads);
    dev.items_per_sm = s.items_per_sm;
    blocked_levels = s.blocked_levels;
    dev.scan_threads = s.scan_threads;
    dev.n_fchunks = (dev.features + s.scan_threads / 32 - 1) / (s.scan_threads / 32);
    reset_graphs();
  }

  // Enqueue one boosting round. Returns the number of kernels enqueued. root_gradient_only:
  // the roots' count and hessian histograms come from the fit's first round.
  uint64_t enqueue_round(bool record_events, bool root_gradient_only) {
    cudaStream_t s = b->stream;
    uint64_t k = 0;
    CK(launch_round_begin(dev, s)); ++k;
    CK(launch_gradients(dev, std::max(1, std::min(grid(4), int((dev.seg_stride + 255) / 256))), s)); ++k;
    CK(launch_round_setup(dev, s)); ++k;
    if (leafwise) {
      k += enqueue_leafwise(root_gradient_only);
      CK(launch_apply_leaves(dev, grid(8), s)); k += 2;
      CK(launch_round_end(dev, s)); ++k;
      return k;
    }
    const uint32_t levels = std::max<uint32_t>(depth, 1);
    for (uint32_t d = 0; d < levels; ++d) {
      const int parity = int(d & 1);
      if (d == 0) {
        CK(launch_zero_build_slots(dev, grid(8), s)); ++k;
      } else {
        CK(cudaStreamWaitEvent(s, zero_ev, 0));  // this level's slots were cleared beside the partition
      }
      if (record_events) CK(cudaEventRecord(events[2 * d], s));
      if (options & MPSB_OPT_PER_NODE) {
        k += enqueue_hist_per_node(d);
      } else {
        TrainerDev view = level_view(d);
        if (d == 0 && root_gradient_only) view.mode = kModeFixedG;
        CK(launch_hist_build(view, hcfg, grid(1), s)); ++k;
      }
      if (record_events) {
        CK(cudaEventRecord(events[2 * d + 1], s));
        CK(cudaMemcpyAsync(level_cells + d, &dev.ctl->cells, sizeof(unsigned long long),
                           cudaMemcpyDeviceToDevice, s));
      }
      if (d == 0) {
        if (root_reuse) {
          CK(launch_root_cache(dev, root_gradient_only ? 0 : 1, grid(4), s)); ++k;
        }
        CK(launch_root_stats(dev, s)); ++k;
      } else if (!dev.fused_sub) {
        CK(launch_subtract(dev, grid(8), s)); ++k;
      }
      if (depth > 0) {
        CK(launch_split_scan(dev, parity, grid(4), s)); k += split_scan_kernels(dev);
      }
      CK(launch_finalize(dev, parity, d, s)); ++k;
      if (d + 1 < depth) {
        // The next level's build slots (named by the finalize) are cleared on the side
        // stream while the partition moves the rows.
        CK(cudaEventRecord(fork_ev, s));
        CK(cudaStreamWaitEvent(side, fork_ev, 0));
        CK(launch_zero_build_slots(dev, grid(8), side)); ++k;
        CK(cudaEventRecord(zero_ev, side));
        CK(launch_partition(dev, grid(4), s)); k += kPartitionKernels;
      }
    }
    CK(launch_apply_leaves(dev, grid(8), s)); k += 2;
    CK(launch_round_end(dev, s)); ++k;
    return k;
  }

  // Leaf-wise round body: the root as a depth-0 level, then lw_steps split steps
  // (select, partition, smaller-child histogram, subtraction, children's split scan,
  // merge), then the leaf segments.
  uint64_t enqueue_leafwise(bool root_gradient_only) {
    cudaStream_t s = b->stream;
    uint64_t k = 0;
    CK(launch_zero_build_slots(dev, grid(8), s)); ++k;
    TrainerDev view = level_view(0);
    if (root_gradient_only) view.mode = kModeFixedG;
    CK(launch_hist_build(view, hcfg, grid(1), s)); ++k;
    if (root_reuse) {
      CK(launch_root_cache(dev, root_gradient_only ? 0 : 1, grid(4), s)); ++k;
    }
    CK(launch_root_stats(dev, s)); ++k;
    if (depth > 0) {
      CK(launch_split_scan(dev, 0, grid(4), s)); k += split_scan_kernels(dev);
    }
    CK(launch_leafwise_init(dev, s)); ++k;
    for (uint32_t step = 0; step < lw_steps && depth > 0; ++step) {
      CK(launch_leafwise_select(dev, s)); ++k;
      CK(launch_partition(dev, grid(4), s)); k += kPartitionKernels;
      CK(launch_zero_build_slots(dev, grid(8), s)); ++k;
      CK(launch_hist_build(build_view(), hcfg, grid(1), s)); ++k;
      CK(launch_subtract(dev, grid(8), s)); ++k;
      CK(launch_split_scan(dev, 1, grid(4), s)); k += split_scan_kernels(dev);
      CK(launch_leafwise_merge(dev, s)); ++k;
    }
    CK(launch_leafwise_finish(dev, s)); ++k;
    return k;
  }

  // The histogram launch's view: unit-hessian fixed-point builds count and gradient limbs.
  TrainerDev build_view() const {
    TrainerDev v = dev;
    if (v.mode == kModeFixed && v.unit_hess) v.mode = kModeFixedCG;
    return v;
  }

  // Dense levels (every row of a node close to the next) read the column-blocked copy of
  // the bins, whose 32-byte block rows are consecutive; sparse levels read the padded
  // row-major copy, whose 128-byte row line serves all feature blocks through L2.
  TrainerDev level_view(uint32_t d) const {
    TrainerDev v = build_view();
    if (d < blocked_levels) {
      v.bins = ds->bins_blocked.as<uint8_t>();
      v.bins_row_stride = kBlockFeatures;
      v.bins_block_stride = uint64_t(ds->n_rows) * kBlockFeatures;
    }
    return v;
  }

  // Plain path: the host reads the level's build list and launches one histogram build
  // per node, waiting for each level (the per-node submit/wait of mps_histogram.mm:62-80).
  uint64_t enqueue_hist_per_node(uint32_t d) {
    cudaStream_t s = b->stream;
    Control c;
    CK(cudaMemcpyAsync(&c, dev.ctl, sizeof c, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<uint32_t> prefix(c.n_build + 1);
    CK(cudaMemcpyAsync(prefix.data(), dev.build_prefix, prefix.size() * sizeof(uint32_t),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    uint64_t k = 0;
    for (uint32_t e = 0; e < c.n_build; ++e) {
      TrainerDev one = level_view(d);
      one.item_begin = prefix[e] * dev.nfb;
      one.item_end = prefix[e + 1] * dev.nfb;
      CK(cudaMemsetAsync(&dev.ctl->hist_counter, 0, sizeof(uint32_t), s));
      CK(launch_hist_build(one, hcfg, grid(1), s));
      ++k;
      CK(cudaStreamSynchronize(s));
    }
    return k;
  }

  void run(uint32_t rounds) {
    b->activate();
    if (rounds_enqueued + rounds > dev.max_rounds)
      throw TrainingError("training session round capacity exceeded");
    const bool timing = (options & MPSB_OPT_TIMING) && !leafwise;  // events are per depth level
    // Events captured into a graph cannot be timed, so timing runs launch directly.
    const bool use_graph = !(options & (MPSB_OPT_NO_GRAPH | MPSB_OPT_PER_NODE | MPSB_OPT_TIMING));
    PhaseTrace capture_trace("run");
    for (uint32_t r = 0; r < rounds; ++r) {
      const bool g_only = root_reuse && root_saved;
      const int gi = g_only ? 1 : 0;
      if (use_graph) {
        if (!graph_exec[gi]) {
          CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
          uint64_t k = 0;
          try {
            k = enqueue_round(timing, g_only);
          } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(b->stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
          }
          CK(cudaStreamEndCapture(b->stream, &graph[gi]));
          CK(cudaGraphInstantiate(&graph_exec[gi], graph[gi], 0));
          kernels_per_round[gi] = k;
          capture_trace.mark(gi ? "capture + instantiate (1)" : "capture + instantiate (0)");
        }
        CK(cudaGraphLaunch(graph_exec[gi], b->stream));
        stats.kernel_launches += kernels_per_round[gi];
      } else {
        stats.kernel_launches += enqueue_round(timing, g_only);
      }
      root_saved = root_reuse;
      stats.hist_launches += (options & MPSB_OPT_PER_NODE) ? 0 : std::max<uint32_t>(depth, 1);
      ++rounds_enqueued;
      ++stats.rounds;
      if (timing) {
        CK(cudaStreamSynchronize(b->stream));
        const uint32_t levels = std::max<uint32_t>(depth, 1);
        std::vector<unsigned long long> after(levels);
        CK(cudaMemcpy(after.data(), level_cells, levels * sizeof(unsigned long long),
                      cudaMemcpyDeviceToHost));
        level_ms.resize(levels, 0.0);
        level_cells_total.resize(levels, 0);
        for (uint32_t d = 0; d < levels; ++d) {
          float ms = 0.0f;
          CK(cudaEventElapsedTime(&ms, events[2 * d], events[2 * d + 1]));
          stats.hist_ms += ms;
          ++stats.hist_timed_launches;
          level_ms[d] += ms;
          level_cells_total[d] += after[d] - (d ? after[d - 1] : cells_before_round);
        }
        cells_before_round = after[levels - 1];
      }
    }
  }

  void synchronize() {
    b->activate();
    CK(cudaStreamSynchronize(b->stream));
    Control c;
    CK(cudaMemcpy(&c, dev.ctl, sizeof c, cudaMemcpyDeviceToHost));
    stats.hist_cells = c.cells - cells_base;
    stats.hist_rows = c.rows_built - rows_base;
    stats.part_rows = c.rows_partitioned - part_base;
    if (c.error) throw TrainingError(describe_device_error(c.error));
  }
};

namespace {

// A batch of forest trees: per tree its sample (a multiset of rows, ascending), feature
// subset (as a mask and ranks), random-threshold seed and base score.
struct ForestSpec {
  uint32_t n_trees = 0;
  uint32_t cap = 0;                  // largest sample
  std::vector<uint32_t> sample;      // [n_trees][cap]
  std::vector<uint32_t> count;       // [n_trees]
  std::vector<uint32_t> masks;       // [n_trees][path_words]
  std::vector<uint32_t> ranks;       // [n_trees][features]
  std::vector<uint32_t> seeds;       // [n_trees] or empty
  std::vector<double> base_scores;   // [n_trees]
};

void setup_trainer(mpsb_cuda_trainer* t, mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                   const double* labels, const double* weights, uint64_t n,
                   const mpsb_train_params* p, uint32_t options, uint32_t n_classes,
                   const ForestSpec* forest = nullptr, uint32_t softmax_classes = 0) {
  if (!b || !ds || !labels || !p) throw TrainingError("null argument");
  PhaseTrace trace("setup");
  validate_training_params(*p);
  validate_tree_params(*p, ds->features);
  if (n != ds->n_rows) throw TrainingError("Training data, labels, or max_bins contract does not match");
  // Weight checks and total; for a single boosted tree of a mean-type objective also the
  // base score's label sum, in the same pass.
  const bool single_mean = !forest && !softmax_classes && n_classes == 0 && label_mode_of(p->objective) != 0;
  const RowSums sums = row_sums(weights, single_mean ? labels : nullptr, n, label_mode_of(p->objective),
                                count_objective_name(p->objective));
  trace.mark("validate weights, label sum");
  // An asynchronous dataset upload ran beside the host passes above.
  dataset_ready(ds);
  trace.mark("dataset upload complete");
  b->activate();
  t->b = b;
  t->ds = ds;
  CK(cudaStreamCreateWithFlags(&t->side, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&t->fork_ev, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&t->zero_ev, cudaEventDisableTiming));
  t->params = *p;
  t->options = options;
  t->depth = p->max_depth;
  t->leafwise = p->growth_strategy == 1;
  if (t->leafwise && (forest || n_classes > 1024))
    throw UnsupportedError("leaf-wise growth on the CUDA backend trains boosting, one-vs-rest (<= 1024 classes) and softmax models");
  t->ovr = n_classes > 0;
  t->n_trees = forest ? forest->n_trees : (t->ovr ? n_classes : 1);
  if (t->ovr && p->objective != MPSB_BINARY_LOGISTIC)
    throw TrainingError("one-vs-rest training uses the binary_logistic objective");
  const uint32_t T = t->n_trees;
  const uint32_t F = ds->features;
  const uint32_t D = p->max_depth;
  if (D > 24) throw UnsupportedError("max_depth above 24 is not supported by the CUDA backend");
  const uint64_t max_leaves_eff = effective_max_leaves(*p);
  const uint64_t seg_rows = forest ? forest->cap : n;  // positions per tree
  const uint64_t by_rows = std::max<uint64_t>(1, (seg_rows + p->min_samples_leaf - 1) / p->min_samples_leaf);
  const uint64_t leaves = std::min<uint64_t>({uint64_t(1) << std::min<uint32_t>(D, 30), max_leaves_eff, by_rows});
  const uint64_t level_nodes = std::max<uint64_t>(1, std::min<uint64_t>(D ? (uint64_t(1) << (D - 1)) : 1, leaves));
  const uint64_t tree_nodes = 2 * leaves + 1;
  TrainerDev& a = t->dev;
  a = TrainerDev{};
  a.bins = ds->bins.as<uint8_t>();
  a.bins_row_stride = uint64_t(ds->nfb) * kBlockFeatures;
  a.bins_block_stride = kBlockFeatures;
  a.bins_fm = ds->bins_fm.as<uint8_t>();
  a.slots = ds->slots;
  // Level-wise growth on u8 datasets: the split scan forms each sibling's histogram
  // (MPSB_FUSED_SUB=0: subtract_kernel does).
  a.fused_sub = ds->slots == uint32_t(kSlots) && p->growth_strategy != 1;
  if (const char* v = std::getenv("MPSB_FUSED_SUB")) a.fused_sub = a.fused_sub && std::atoi(v) != 0;
  a.bins16 = ds->bins16.as<uint16_t>();
  a.bins16_fm = ds->bins16_fm.as<uint16_t>();
  a.bin_count = ds->bin_count.as<uint32_t>();
  a.sm_count = uint32_t(b->sm_count);
  a.has_missing = ds->has_missing.as<uint8_t>();
  a.n_rows = ds->n_rows;
  a.seg_stride = uint32_t(seg_rows);
  a.features = F;
  a.nfb = ds->nfb;
  a.n_trees = T;
  a.objective = p->objective;
  a.ovr = t->ovr ? 1 : 0;
  a.n_classes = softmax_classes;
  t->softmax_classes = softmax_classes;
  a.mode = (options & MPSB_OPT_FLOAT_HIST) ? kModeFloat : kModeFixed;
  // Four features (warps) per split-scan CTA spread a shallow level's few nodes over many
  // SMs; MPSB_SCAN_THREADS overrides (a multiple of 32, at most 512).
  a.scan_threads = 128;
  // rows per histogram work item: chosen per level on the device (about three items per
  // SM, within the 2^16-row limb bound)
  a.item_rows = 0;
  // Squared error and quantile have h = 1 per row; without weights every row's quantized
  // hessian is the same unit (MPSB_UNIT_HESS=0 builds the hessian limbs anyway).
  a.unit_hess = !softmax_classes && n_classes == 0 && unit_hessian_fit(weights, *p);
  {
    // A shape the autotuner chose for this kind of fit.
    mpsb_cuda_tuning tuned{};
    if (!forest && !softmax_classes && n_classes == 0 &&
        tuned_shape(tune_key_of(ds, weights, *p, options), &tuned)) {
      t->hcfg.threads = int(tuned.hist_threads);
      t->hcfg.stages = int(tuned.hist_stages);
      t->hcfg.root_threads = int(tuned.root_threads);
      a.items_per_sm = tuned.items_per_sm;
      t->blocked_levels = tuned.blocked_levels;
      a.scan_threads = tuned.scan_threads;
    }
  }
  t->hcfg.bins_tmap = ds->has_bins_tmap ? &ds->bins_tmap : nullptr;
  // Launch-shape overrides (tuning sweeps): threads per CTA, pipeline stages, rows per work
  // item, split-scan CTA size.
  if (const char* v = std::getenv("MPSB_SCAN_THREADS"))
    a.scan_threads = uint32_t(std::min(512, std::max(32, std::atoi(v) / 32 * 32)));
  a.n_fchunks = (F + a.scan_threads / 32 - 1) / (a.scan_threads / 32);
  if (const char* v = std::getenv("MPSB_HIST_THREADS")) t->hcfg.threads = std::atoi(v);
  if (const char* v = std::getenv("MPSB_HIST_STAGES")) t->hcfg.stages = std::atoi(v);
  t->hcfg.direct = true;
  if (const char* v = std::getenv("MPSB_HIST_DIRECT")) t->hcfg.direct = std::atoi(v) != 0;
  if (const char* v = std::getenv("MPSB_ROOT_THREADS")) t->hcfg.root_threads = std::atoi(v);
  if (const char* v = std::getenv("MPSB_WIDE_THREADS")) t->hcfg.wide_threads = std::atoi(v);
  if (const char* v = std::getenv("MPSB_BLOCKED_LEVELS")) t->blocked_levels = uint32_t(std::atoi(v));
  if (const char* v = std::getenv("MPSB_ITEMS_PER_SM")) a.items_per_sm = uint32_t(std::max(1, std::atoi(v)));
  if (const char* v = std::getenv("MPSB_ITEM_ROWS"))
    a.item_rows = uint32_t(std::min<long>(std::max<long>(std::atol(v), 512), long(kItemRowsMax)));
  // Squared error and quantile have hessian = sample weight, the same in every round: the
  // roots' count and hessian histograms are built once per fit (MPSB_ROOT_REUSE=0 builds
  // them every round).
  t->root_reuse = !forest && !softmax_classes && a.mode == kModeFixed && !(options & MPSB_OPT_PER_NODE) &&
                  (p->objective == MPSB_SQUARED_ERROR || p->objective == MPSB_QUANTILE);
  if (const char* v = std::getenv("MPSB_ROOT_REUSE")) t->root_reuse = t->root_reuse && std::atoi(v) != 0;
  if (t->root_reuse) {
    a.root_cache = t->alloc<unsigned long long>(size_t(T) * F * ds->slots * 2);
    a.root_cache_kh = t->alloc<int>(T);
  }
  TreeParams& tp = a.params;
  tp.min_samples_leaf = p->min_samples_leaf;
  tp.min_child_weight = p->min_child_weight;
  tp.reg_lambda = p->reg_lambda;
  tp.reg_alpha = p->reg_alpha;
  tp.max_delta_step = p->max_delta_step;
  tp.gamma = p->gamma;
  tp.min_gain_to_split = p->min_gain_to_split;
  tp.learning_rate = p->learning_rate;
  tp.max_depth = D;
  tp.max_leaves = uint32_t(std::min<uint64_t>(max_leaves_eff, 0xFFFFFFFFull));
  tp.split_strategy = p->split_strategy;
  tp.random_seed = p->random_seed;
  tp.has_monotonic = p->n_monotonic ? 1 : 0;
  tp.n_groups = p->n_interaction_groups;
  tp.path_words = (F + 31) / 32;
  tp.objective = p->objective;
  tp.objective_alpha = p->objective_alpha;
  tp.tweedie_variance_power = p->tweedie_variance_power;
  set_screen_constants(tp);
  cudaStream_t s = b->stream;
  const uint32_t W = tp.path_words;

  trace.mark("parameters, root cache");
  // inputs
  double* d_labels = t->alloc<double>(n);
  CK(cudaMemcpyAsync(d_labels, labels, n * sizeof(double), cudaMemcpyHostToDevice, s));
  a.labels = d_labels;
  if (weights) {
    double* d_w = t->alloc<double>(n);
    CK(cudaMemcpyAsync(d_w, weights, n * sizeof(double), cudaMemcpyHostToDevice, s));
    a.weights = d_w;
  }

  if (softmax_classes) {
    // Margins [K][n] from the class priors (WeightedClassBaseScores,
    // multiclass_trainer.cpp:39-67); labels must be class ids (22-37).
    const uint32_t K = softmax_classes;
    const double total = sums.total;
    std::vector<double> cw(K, 0.0);
    for (uint64_t i = 0; i < n; ++i) {
      const double y = labels[i];
      if (!std::isfinite(y)) throw TrainingError("softmax labels must be finite");
      if (std::floor(y) != y || y < 0.0 || y >= double(K))
        throw TrainingError("softmax labels must be encoded class ids");
      cw[uint32_t(y)] += weights ? weights[i] : 1.0;
      if (!std::isfinite(cw[uint32_t(y)])) throw TrainingError("softmax class prior overflowed");
    }
    t->base_scores.resize(K);
    for (uint32_t k = 0; k < K; ++k) {
      t->base_scores[k] = std::log(std::max(1e-15, cw[k] / total));
      if (!std::isfinite(t->base_scores[k])) throw TrainingError("softmax base score is not finite");
    }
    a.preds = t->alloc<double>(size_t(K) * n);
    for (uint32_t k = 0; k < K; ++k) CK(launch_fill_f64(a.preds + size_t(k) * n, n, t->base_scores[k], s));
  }
  trace.mark("label/weight upload");
  if (!softmax_classes) t->base_scores.resize(T);
  if (!softmax_classes) a.preds = t->alloc<double>(size_t(T) * n);
  for (uint32_t k = 0; k < T && !softmax_classes; ++k) {
    t->base_scores[k] = forest ? forest->base_scores[k]
                               : base_score(*p, labels, weights, n, t->ovr ? int64_t(k) : -1, &sums);
    CK(launch_fill_f64(a.preds + size_t(k) * n, n, t->base_scores[k], s));
  }
  trace.mark("base scores, predictions");
  if (p->n_monotonic) {
    int8_t* m = t->alloc<int8_t>(F);
    CK(cudaMemcpyAsync(m, p->monotonic_constraints, F, cudaMemcpyHostToDevice, s));
    a.monotonic = m;
  }
  if (p->n_interaction_groups) {
    std::vector<uint32_t> masks(size_t(p->n_interaction_groups) * W, 0);
    for (uint32_t g = 0; g < p->n_interaction_groups; ++g)
      for (uint32_t i = p->interaction_offsets[g]; i < p->interaction_offsets[g + 1]; ++i) {
        const uint32_t f = p->interaction_features[i];
        masks[size_t(g) * W + f / 32] |= 1u << (f % 32);
      }
    uint32_t* gm = t->alloc<uint32_t>(masks.size());
    CK(cudaMemcpyAsync(gm, masks.data(), masks.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    a.group_masks = gm;
  }
  if (forest) {
    const size_t cells = size_t(T) * forest->cap;
    uint32_t* d_sample = t->alloc<uint32_t>(cells);
    CK(cudaMemcpyAsync(d_sample, forest->sample.data(), cells * 4, cudaMemcpyHostToDevice, s));
    uint32_t* d_count = t->alloc<uint32_t>(T);
    CK(cudaMemcpyAsync(d_count, forest->count.data(), size_t(T) * 4, cudaMemcpyHostToDevice, s));
    uint32_t* d_masks = t->alloc<uint32_t>(size_t(T) * W);
    CK(cudaMemcpyAsync(d_masks, forest->masks.data(), size_t(T) * W * 4, cudaMemcpyHostToDevice, s));
    uint32_t* d_ranks = t->alloc<uint32_t>(size_t(T) * F);
    CK(cudaMemcpyAsync(d_ranks, forest->ranks.data(), size_t(T) * F * 4, cudaMemcpyHostToDevice, s));
    a.sample_rows = d_sample;
    a.sample_count = d_count;
    a.tree_feature_masks = d_masks;
    a.feature_rank = d_ranks;
    if (!forest->seeds.empty()) {
      uint32_t* d_seeds = t->alloc<uint32_t>(T);
      CK(cudaMemcpyAsync(d_seeds, forest->seeds.data(), size_t(T) * 4, cudaMemcpyHostToDevice, s));
      a.tree_seeds = d_seeds;
    }
    a.skip_apply = 1;
    CK(cudaStreamSynchronize(s));
  }
  // working state
  a.gh = t->alloc<float2>(size_t(T) * 2 * seg_rows);
  a.gh_ordered = 1;
  a.rows = t->alloc<uint32_t>(size_t(T) * 2 * seg_rows);
  a.trees = t->alloc<TreeState>(T);
  a.max_level_nodes = uint32_t(T * level_nodes);
  a.n_slots = a.max_level_nodes;
  if (t->leafwise) {
    // Active leaves <= leaves; each active leaf above max_depth keeps a histogram slot
    // from its tree's stack (slot t is the root's).
    const uint64_t max_active = p->max_active_leaves ? p->max_active_leaves : max_leaves_eff;
    a.lw_max_leaves = uint32_t(std::min<uint64_t>(max_leaves_eff, 0xFFFFFFFFull));
    a.lw_max_active = uint32_t(std::min<uint64_t>(max_active, 0xFFFFFFFFull));
    a.lw_cap = uint32_t(std::min<uint64_t>(max_active, leaves) + 2);
    a.lw_slot_cap = uint32_t(std::min<uint64_t>(max_active, leaves) + 1);
    a.n_slots = T + T * a.lw_slot_cap;
    a.max_level_nodes = std::max<uint32_t>(a.max_level_nodes, 2 * T);
    a.lw_active = t->alloc<LeafActive>(size_t(T) * a.lw_cap);
    a.lw_path = t->alloc<uint32_t>(size_t(T) * a.lw_cap * W);
    a.lw_allowed = t->alloc<uint32_t>(size_t(T) * a.lw_cap * W);
    a.lw_count = t->alloc<uint32_t>(T);
    a.lw_done = t->alloc<uint32_t>(T);
    a.lw_slots = t->alloc<uint32_t>(size_t(T) * a.lw_slot_cap);
    a.lw_slot_top = t->alloc<uint32_t>(T);
    a.lw_scan_map = t->alloc<uint32_t>(2 * size_t(T));
    t->lw_steps = uint32_t(leaves > 0 ? leaves - 1 : 0);
  }
  const uint64_t slot_words = uint64_t(F) * ds->slots * 3;
  a.hist = t->alloc<unsigned long long>(uint64_t(a.n_slots) * slot_words);
  a.free_stack = t->alloc<uint32_t>(a.n_slots);
  for (int q = 0; q < 2; ++q) {
    a.nodes[q] = t->alloc<NodeRec>(a.max_level_nodes);
    a.node_path[q] = t->alloc<uint32_t>(size_t(a.max_level_nodes) * W);
    a.node_allowed[q] = t->alloc<uint32_t>(size_t(a.max_level_nodes) * W);
  }
  a.partial = t->alloc<SplitRec>(size_t(a.max_level_nodes) * a.n_fchunks);
  a.node_screen = t->alloc<uint32_t>(a.max_level_nodes);
  a.chunk_screen = t->alloc<uint32_t>(size_t(a.max_level_nodes) * a.n_fchunks);
  a.scan_two_phase = p->split_strategy == 0 && p->reg_alpha == 0.0 && p->reg_lambda > 0.0;
  a.build = t->alloc<BuildEntry>(a.max_level_nodes);
  a.build_prefix = t->alloc<uint32_t>(a.max_level_nodes + 1);
  a.sub = t->alloc<SubEntry>(a.max_level_nodes);
  a.part = t->alloc<PartEntry>(a.max_level_nodes);
  a.part_prefix = t->alloc<uint32_t>(a.max_level_nodes + 1);
  a.max_part_chunks = uint32_t(T * ((seg_rows + kPartChunk - 1) / kPartChunk + level_nodes + 1));
  a.part_counts = t->alloc<uint32_t>(a.max_part_chunks);
  a.part_offsets = t->alloc<uint32_t>(a.max_part_chunks);
  a.part_flags = t->alloc<uint32_t>(size_t(a.max_part_chunks) * (kPartChunk / 32));
  a.max_leafsegs = uint32_t(T * (leaves + 1));
  a.leafseg = t->alloc<LeafSeg>(a.max_leafsegs);
  a.leaf_prefix = t->alloc<uint32_t>(a.max_leafsegs + 1);
  if (!a.skip_apply) {
    a.leaf_of = t->alloc<uint32_t>(size_t(T) * n);
    CK(cudaMemsetAsync(a.leaf_of, 0xff, size_t(T) * n * sizeof(uint32_t), s));  // no leaf yet
    a.leaf_steps = t->alloc<double>(2 * size_t(a.max_leafsegs));
  }
  a.max_tree_nodes = uint32_t(tree_nodes);
  a.tree_nodes = t->alloc<TreeNodeOut>(size_t(T) * tree_nodes);
  a.ctl = t->alloc<Control>(1);
  CK(cudaMemsetAsync(a.ctl, 0, sizeof(Control), s));
  a.scratch_flags = t->alloc<uint32_t>(a.max_level_nodes);
  a.scratch_prefix = t->alloc<uint32_t>(a.max_level_nodes);
  a.scratch_aux = t->alloc<uint32_t>(a.max_level_nodes);
  a.tree_scratch = t->alloc<uint32_t>(size_t(T) * 4);
  a.max_rounds = p->n_estimators * (softmax_classes ? softmax_classes : 1);
  a.model_nodes = t->alloc<TreeNodeOut>(size_t(a.max_rounds) * T * tree_nodes);
  a.model_counts = t->alloc<uint32_t>(size_t(a.max_rounds) * T);
  a.round_counter = t->alloc<uint32_t>(1);
  CK(cudaMemsetAsync(a.round_counter, 0, sizeof(uint32_t), s));
  a.item_begin = a.item_end = 0;
  if (options & MPSB_OPT_TIMING) {
    t->events.resize(2 * std::max<uint32_t>(D, 1));
    for (auto& e : t->events) CK(cudaEventCreate(&e));
    t->level_cells = t->alloc<unsigned long long>(std::max<uint32_t>(D, 1));
  }
  CK(cudaStreamSynchronize(s));
  trace.mark("working state");
}

mpsb_cuda_model* export_model(mpsb_cuda_trainer* t, uint32_t tree_index,
                              bool with_predictions = true) {
  const TrainerDev& a = t->dev;
  PhaseTrace trace("export");
  uint32_t rounds = 0;
  CK(cudaMemcpy(&rounds, a.round_counter, sizeof rounds, cudaMemcpyDeviceToHost));
  std::vector<uint32_t> counts(size_t(rounds) * a.n_trees);
  if (!counts.empty())
    CK(cudaMemcpy(counts.data(), a.model_counts, counts.size() * 4, cudaMemcpyDeviceToHost));
  std::unique_ptr<mpsb_cuda_model> m(new mpsb_cuda_model);
  m->base = t->base_scores[tree_index];
  m->learning_rate = t->params.learning_rate;
  m->objective = t->params.objective;
  m->objective_alpha = t->params.objective_alpha;
  m->tweedie_variance_power = t->params.tweedie_variance_power;
  const mpsb_cuda_dataset* ds = t->ds;
  if (ds->has_schema) {  // a device-quantized dataset carries the file's schema
    m->has_schema = true;
    m->features = ds->features;
    m->max_bins = ds->max_bins;
    m->boundaries = ds->boundaries;
    m->boundary_offset = ds->boundary_offset;
    m->boundary_count = ds->boundary_count;
    m->bin_count = ds->h_bin_count;
    m->missing_count = ds->missing_count;
  }
  m->n_trees = rounds;
  m->trees.resize(rounds);
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t c = counts[size_t(r) * a.n_trees + tree_index];
    m->trees[r].resize(c);
    CK(cudaMemcpy(m->trees[r].data(),
                  a.model_nodes + (size_t(r) * a.n_trees + tree_index) * a.max_tree_nodes,
                  size_t(c) * sizeof(mpsb_tree_node), cudaMemcpyDeviceToHost));
  }
  trace.mark("trees");
  if (with_predictions) {
    const size_t bytes = size_t(a.n_rows) * sizeof(double);
    m->device_predictions.alloc(bytes);
    m->device_prediction_count = a.n_rows;
    m->device = t->b->device;
    CK(cudaMemcpyAsync(m->device_predictions.p, a.preds + size_t(tree_index) * a.n_rows, bytes,
                       cudaMemcpyDeviceToDevice, t->b->stream));
    CK(cudaStreamSynchronize(t->b->stream));
    trace.mark("prediction copy (device)");
  }
  return m.release();
}

// A softmax model: K base scores, the trees of every (round, class) in that order, and
// the training margins [rows][K].
mpsb_cuda_model* export_softmax(mpsb_cuda_trainer* t) {
  mpsb_cuda_model* m = export_model(t, 0, false);
  const uint32_t K = t->softmax_classes;
  const TrainerDev& a = t->dev;
  m->class_count = K;
  m->base_scores = t->base_scores;
  m->base = 0.0;
  m->class_labels.resize(K);
  for (uint32_t k = 0; k < K; ++k) m->class_labels[k] = double(k);
  std::vector<double> margins(size_t(K) * a.n_rows);
  CK(cudaMemcpy(margins.data(), a.preds, margins.size() * sizeof(double), cudaMemcpyDeviceToHost));
  m->train_predictions.resize(margins.size());
  for (uint32_t k = 0; k < K; ++k)
    for (uint32_t r = 0; r < a.n_rows; ++r)
      m->train_predictions[size_t(r) * K + k] = margins[size_t(k) * a.n_rows + r];
  return m;
}

static_assert(sizeof(mpsb_tree_node) == sizeof(TreeNodeOut), "tree node layout");

}  // namespace

extern "C" {

int mpsb_cuda_trainer_create(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                             const double* labels, const double* weights, uint64_t n,
                             const mpsb_train_params* p, uint32_t options,
                             mpsb_cuda_trainer** out) {
  return guard([&] {
    std::unique_ptr<mpsb_cuda_trainer> t(new mpsb_cuda_trainer);
    setup_trainer(t.get(), b, ds, labels, weights, n, p, options, 0);
    *out = t.release();
  });
}

int mpsb_cuda_trainer_run(mpsb_cuda_trainer* t, uint32_t rounds) {
  return guard([&] { t->run(rounds); });
}

int mpsb_cuda_trainer_synchronize(mpsb_cuda_trainer* t) {
  return guard([&] { t->synchronize(); });
}

int mpsb_cuda_trainer_stats(const mpsb_cuda_trainer* t, mpsb_cuda_stats* out) {
  return guard([&] { *out = t->stats; });
}

int mpsb_cuda_trainer_reset_stats(mpsb_cuda_trainer* t) {
  return guard([&] {
    t->synchronize();
    Control c;
    CK(cudaMemcpy(&c, t->dev.ctl, sizeof c, cudaMemcpyDeviceToHost));
    t->cells_base = c.cells;
    t->rows_base = c.rows_built;
    t->part_base = c.rows_partitioned;
    t->cells_before_round = c.cells;
    t->stats = mpsb_cuda_stats{};
    t->level_ms.assign(t->level_ms.size(), 0.0);
    t->level_cells_total.assign(t->level_cells_total.size(), 0);
  });
}

int mpsb_cuda_trainer_level_stats(const mpsb_cuda_trainer* t, uint32_t n_levels, double* ms,
                                  uint64_t* cells) {
  return guard([&] {
    for (uint32_t d = 0; d < n_levels; ++d) {
      ms[d] = d < t->level_ms.size() ? t->level_ms[d] : 0.0;
      cells[d] = d < t->level_cells_total.size() ? t->level_cells_total[d] : 0;
    }
  });
}

int mpsb_cuda_trainer_export(mpsb_cuda_trainer* t, mpsb_cuda_model** out) {
  return guard([&] {
    t->synchronize();
    *out = export_model(t, 0);
  });
}

void mpsb_cuda_trainer_destroy(mpsb_cuda_trainer* t) { delete t; }

int mpsb_cuda_autotune(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds, const double* labels,
                       const double* weights, uint64_t n, const mpsb_train_params* p,
                       uint32_t options, uint32_t rounds_per_trial, mpsb_cuda_tuning* out) {
  return guard([&] {
    if (!b || !ds || !labels || !p || !out) throw TrainingError("null argument");
    dataset_ready(ds);
    if (options & (MPSB_OPT_PER_NODE | MPSB_OPT_TIMING | MPSB_OPT_NO_GRAPH))
      throw UnsupportedError("the autotuner times the batched, graph-captured rounds");
    const uint32_t R = std::max(1u, rounds_per_trial);
    constexpr uint32_t kMaxTrials = 16, kConfirmTrials = 4;
    mpsb_train_params tp = *p;
    tp.n_estimators = (kMaxTrials + kConfirmTrials) * (R + 1) + 1;
    std::unique_ptr<mpsb_cuda_trainer> t(new mpsb_cuda_trainer);
    const TuneKey key = tune_key_of(ds, weights, *p, options);
    {
      // The session starts from the built-in shape, not from an earlier tuning.
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      g_tune_table.erase(key);
    }
    setup_trainer(t.get(), b, ds, labels, weights, n, &tp, options, 0);
    mpsb_cuda_tuning cur{};
    cur.hist_threads = uint32_t(t->hcfg.threads);
    cur.hist_stages = uint32_t(t->hcfg.stages);
    cur.root_threads = uint32_t(t->hcfg.root_threads);
    cur.items_per_sm = t->dev.items_per_sm ? t->dev.items_per_sm : 3u;
    cur.blocked_levels = t->blocked_levels;
    cur.scan_threads = t->dev.scan_threads;
    const uint32_t min_scan = t->dev.scan_threads;  // the chunk tables are sized for it
    const mpsb_cuda_tuning built_in_shape = cur;
    auto same_shape = [](const mpsb_cuda_tuning& x, const mpsb_cuda_tuning& y) {
      return x.hist_threads == y.hist_threads && x.hist_stages == y.hist_stages &&
             x.root_threads == y.root_threads && x.items_per_sm == y.items_per_sm &&
             x.blocked_levels == y.blocked_levels && x.scan_threads == y.scan_threads;
    };
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    uint32_t trials = 0;
    auto measure = [&](const mpsb_cuda_tuning& s) -> double {
      t->apply_shape(s);
      t->run(1);  // captures the round graphs of this shape (and the roots' reuse)
      CK(cudaEventRecord(e0, b->stream));
      t->run(R);
      CK(cudaEventRecord(e1, b->stream));
      t->synchronize();
      float ms = 0.0f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      ++trials;
      return double(ms) / R;
    };
    try {
      double best = measure(cur);
      const double built_in = best;
      // Coordinate descent over the shape, one parameter at a time.
      auto try_values = [&](auto set, std::initializer_list<uint32_t> values) {
        for (uint32_t v : values) {
          if (trials >= kMaxTrials) return;
          mpsb_cuda_tuning cand = cur;
          if (!set(cand, v)) continue;
          const double ms = measure(cand);
          if (ms < best) {
            best = ms;
            cur = cand;
          }
        }
      };
      try_values([&](mpsb_cuda_tuning& c, uint32_t v) {
        if (v == c.hist_threads) return false;
        c.hist_threads = v;
        c.hist_stages = 2;
        return true;
      }, {768, 640, 512});
      try_values([&](mpsb_cuda_tuning& c, uint32_t v) {
        if (c.hist_threads != 512 || v == c.hist_stages) return false;
        c.hist_stages = v;
        return true;
      }, {3});
      try_values([&](mpsb_cuda_tuning& c, uint32_t v) {
        if (v == c.items_per_sm) return false;
        c.items_per_sm = v;
        return true;
      }, {2, 3, 4});
      try_values([&](mpsb_cuda_tuning& c, uint32_t v) {
        if (v == c.blocked_levels) return false;
        c.blocked_levels = v;
        return true;
      }, {1, 2, 3});
      try_values([&](mpsb_cuda_tuning& c, uint32_t v) {
        if (v == c.scan_threads || v < min_scan) return false;
        c.scan_threads = v;
        return true;
      }, {128, 256});
      try_values([&](mpsb_cuda_tuning& c, uint32_t v) {
        if (v == c.root_threads) return false;
        c.root_threads = v;
        return true;
      }, {1024, 768});
      // Rounds differ a little from tree to tree: confirm the winner against the built-in
      // shape with alternating measurements before keeping it.
      mpsb_cuda_tuning chosen = cur;
      double chosen_ms = best, default_ms = built_in;
      if (!same_shape(cur, built_in_shape)) {
        double d = 0.0, c = 0.0;
        for (uint32_t i = 0; i < kConfirmTrials / 2; ++i) {
          d += measure(built_in_shape);
          c += measure(cur);
        }
        default_ms = d / (kConfirmTrials / 2);
        chosen_ms = c / (kConfirmTrials / 2);
        if (!(chosen_ms < default_ms)) {
          chosen = built_in_shape;
          chosen_ms = default_ms;
        }
      }
      cur = chosen;
      cur.ms_per_round = chosen_ms;
      cur.default_ms_per_round = default_ms;
      cur.trials = trials;
    } catch (...) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    {
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      g_tune_table[key] = cur;
    }
    *out = cur;
  });
}

void mpsb_cuda_autotune_clear(void) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune_table.clear();
}

int mpsb_cuda_train_regressor(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                              const double* labels, const double* weights, uint64_t n,
                              const mpsb_train_params* p, uint32_t options,
                              mpsb_cuda_model** out) {
  return guard([&] {
    std::unique_ptr<mpsb_cuda_trainer> t(new mpsb_cuda_trainer);
    setup_trainer(t.get(), b, ds, labels, weights, n, p, options, 0);
    t->run(p->n_estimators);
    t->synchronize();
    *out = export_model(t.get(), 0);
  });
}

int mpsb_cuda_train_ovr(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                        const double* labels, const double* weights, uint64_t n,
                        uint32_t n_classes, const mpsb_train_params* p, uint32_t options,
                        mpsb_cuda_model** out) {
  return guard([&] {
    if (n_classes < 2) throw TrainingError("one-vs-rest needs at least two classes");
    for (uint64_t i = 0; i < n; ++i) {
      const double y = labels[i];
      if (!(y >= 0.0 && y < double(n_classes) && std::floor(y) == y))
        throw TrainingError("one-vs-rest labels must be class ids in [0, n_classes)");
    }
    std::unique_ptr<mpsb_cuda_trainer> t(new mpsb_cuda_trainer);
    setup_trainer(t.get(), b, ds, labels, weights, n, p, options, n_classes);
    t->run(p->n_estimators);
    t->synchronize();
    for (uint32_t k = 0; k < n_classes; ++k) out[k] = export_model(t.get(), k);
  });
}

int mpsb_cuda_train_softmax(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                            const double* labels, const double* weights, uint64_t n,
                            const mpsb_train_params* p, uint32_t class_count, uint32_t options,
                            mpsb_cuda_model** out) {
  return guard([&] {
    if (!out) throw TrainingError("null argument");
    if (class_count < 2) throw TrainingError("softmax class_count must be at least two");
    std::unique_ptr<mpsb_cuda_trainer> t(new mpsb_cuda_trainer);
    setup_trainer(t.get(), b, ds, labels, weights, n, p, options, 0, nullptr, class_count);
    t->run(p->n_estimators * class_count);
    t->synchronize();
    *out = export_softmax(t.get());
  });
}

int mpsb_cuda_train_forest(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                           const double* labels, const double* weights, uint64_t n,
                           const mpsb_train_params* p, uint32_t n_trees,
                           const uint8_t* row_counts, const uint32_t* feature_offsets,
                           const uint32_t* features, const uint32_t* seeds, uint32_t options,
                           mpsb_cuda_model** out) {
  return guard([&] {
    if (!b || !ds || !labels || !p || !row_counts || !feature_offsets || !features || !out)
      throw TrainingError("null argument");
    if (n_trees == 0) throw TrainingError("n_estimators must be at least 1");
    if (n != ds->n_rows) throw TrainingError("Training data, labels, or max_bins contract does not match");
    if (p->n_interaction_groups)
      throw UnsupportedError("forest training on the CUDA backend takes no interaction constraints");
    validate_training_params(*p);
    validate_tree_params(*p, ds->features);
    validate_weights(weights, n);
    const uint32_t F = ds->features, W = (F + 31) / 32;
    // Trees per trainer: the histogram slots of a tree's widest level dominate its device
    // memory, so batch as many trees as fit in half of the free memory.
    mpsb_train_params tp = *p;
    tp.n_estimators = 1;
    // Sample sizes of every tree (independent trees: worker threads).
    std::vector<uint64_t> sample_size(n_trees, 0);
    parallel_trees(n_trees, [&](uint32_t t) {
      uint64_t c = 0;
      const uint8_t* m = row_counts + size_t(t) * n;
      for (uint64_t r = 0; r < n; ++r) c += m[r];
      sample_size[t] = c;
    });
    uint64_t cap_all = 1;
    for (uint32_t t = 0; t < n_trees; ++t) {
      const uint64_t c = sample_size[t];
      if (c == 0) throw TrainingError("a forest tree's row sample must not be empty");
      if (c >= 0x80000000ull) throw UnsupportedError("a forest tree's row sample exceeds 2^31 rows");
      cap_all = std::max(cap_all, c);
      const uint32_t f0 = feature_offsets[t], f1 = feature_offsets[t + 1];
      if (f1 <= f0) throw TrainingError("a forest tree's feature subset must not be empty");
      std::vector<uint8_t> seen(F, 0);
      for (uint32_t i = f0; i < f1; ++i) {
        if (features[i] >= F) throw TrainingError("forest feature index out of range");
        if (seen[features[i]]++) throw TrainingError("forest feature subsets must not repeat a feature");
      }
    }
    const uint64_t leaves = std::min<uint64_t>(
        {uint64_t(1) << std::min<uint32_t>(p->max_depth, 30), std::max<uint64_t>(effective_max_leaves(*p), 2),
         std::max<uint64_t>(1, (cap_all + p->min_samples_leaf - 1) / p->min_samples_leaf)});
    const uint64_t per_tree = leaves * uint64_t(F) * ds->slots * 24 + cap_all * (2 * 12 + 8) + n * 8 +
                              uint64_t(2 * leaves + 1) * 64 * 8;
    size_t free_b = 0, total_b = 0;
    b->activate();
    CK(cudaMemGetInfo(&free_b, &total_b));
    uint64_t batch = std::max<uint64_t>(1, (free_b / 2) / std::max<uint64_t>(per_tree, 1));
    if (const char* v = std::getenv("MPSB_FOREST_BATCH")) batch = std::max(1, std::atoi(v));
    batch = std::min<uint64_t>(batch, n_trees);
    for (uint32_t t0 = 0; t0 < n_trees; t0 += uint32_t(batch)) {
      const uint32_t B = std::min<uint32_t>(uint32_t(batch), n_trees - t0);
      ForestSpec fs;
      fs.n_trees = B;
      fs.count.resize(B);
      for (uint32_t k = 0; k < B; ++k) {
        fs.count[k] = uint32_t(sample_size[t0 + k]);
        fs.cap = std::max<uint32_t>(fs.cap, fs.count[k]);
      }
      fs.sample.assign(size_t(B) * fs.cap, 0);
      fs.masks.assign(size_t(B) * W, 0);
      fs.ranks.assign(size_t(B) * F, 0);
      fs.base_scores.resize(B);
      if (seeds) fs.seeds.assign(seeds + t0, seeds + t0 + B);
      const int mode = label_mode_of(tp.objective);
      parallel_trees(B, [&](uint32_t k) {
        const uint8_t* m = row_counts + size_t(t0 + k) * n;
        uint32_t* dst = fs.sample.data() + size_t(k) * fs.cap;
        uint32_t pos = 0;
        for (uint64_t r = 0; r < n; ++r)
          for (uint32_t c = 0; c < m[r]; ++c) dst[pos++] = uint32_t(r);
        // The reference fits the tree on its sample: base score over the sample's rows in
        // order (each row as often as it was drawn).
        if (mode) {
          fs.base_scores[k] = multiset_base_score(tp, labels, weights, m, n, mode);
        } else {
          std::vector<double> ys, ws;
          ys.reserve(pos);
          if (weights) ws.reserve(pos);
          for (uint32_t i = 0; i < pos; ++i) {
            ys.push_back(labels[dst[i]]);
            if (weights) ws.push_back(weights[dst[i]]);
          }
          fs.base_scores[k] = base_score(tp, ys.data(), weights ? ws.data() : nullptr, ys.size(), -1);
        }
        std::vector<uint32_t> sub(features + feature_offsets[t0 + k], features + feature_offsets[t0 + k + 1]);
        std::sort(sub.begin(), sub.end());
        for (uint32_t i = 0; i < sub.size(); ++i) {
          fs.masks[size_t(k) * W + sub[i] / 32] |= 1u << (sub[i] % 32);
          fs.ranks[size_t(k) * F + sub[i]] = i;  // position in the tree's ascending subset
        }
      });
      std::unique_ptr<mpsb_cuda_trainer> t(new mpsb_cuda_trainer);
      setup_trainer(t.get(), b, ds, labels, weights, n, &tp, options | MPSB_OPT_NO_GRAPH, 0, &fs);
      t->run(1);
      t->synchronize();
      for (uint32_t k = 0; k < B; ++k) out[t0 + k] = export_model(t.get(), k, false);
    }
  });
}

int mpsb_cuda_model_create(double base, double lr, uint32_t n_trees, const uint32_t* counts,
                           const mpsb_tree_node* nodes, mpsb_cuda_model** out) {
  return guard([&] {
    if (!std::isfinite(base) || !std::isfinite(lr) || lr <= 0.0 || lr > 1.0)
      throw TrainingError("Model base score, learning rate, or tree count is invalid");
    std::unique_ptr<mpsb_cuda_model> m(new mpsb_cuda_model);
    m->base = base;
    m->learning_rate = lr;
    m->n_trees = n_trees;
    m->trees.resize(n_trees);
    size_t k = 0;
    for (uint32_t t = 0; t < n_trees; ++t) {
      if (counts[t] == 0) throw TrainingError("Tree model has no root node");
      m->trees[t].assign(nodes + k, nodes + k + counts[t]);
      k += counts[t];
    }
    *out = m.release();
  });
}

uint32_t mpsb_cuda_model_tree_count(const mpsb_cuda_model* m) { return m->n_trees; }
double mpsb_cuda_model_base_score(const mpsb_cuda_model* m) { return m->base; }
double mpsb_cuda_model_learning_rate(const mpsb_cuda_model* m) { return m->learning_rate; }
uint32_t mpsb_cuda_model_tree_node_count(const mpsb_cuda_model* m, uint32_t t) {
  return t < m->trees.size() ? uint32_t(m->trees[t].size()) : 0;
}
int mpsb_cuda_model_tree_nodes(const mpsb_cuda_model* m, uint32_t t, mpsb_tree_node* out) {
  return guard([&] {
    if (t >= m->trees.size()) throw TrainingError("tree index out of range");
    std::memcpy(out, m->trees[t].data(), m->trees[t].size() * sizeof(mpsb_tree_node));
  });
}
int mpsb_cuda_model_train_predictions(const mpsb_cuda_model* m, double* out) {
  return guard([&] {
    if (m->device_prediction_count) {
      CK(cudaSetDevice(m->device));
      CK(cudaMemcpy(out, m->device_predictions.p, m->device_prediction_count * sizeof(double),
                    cudaMemcpyDeviceToHost));
      return;
    }
    if (m->train_predictions.empty())
      throw TrainingError("this model holds no training predictions (forest tree or loaded model)");
    std::memcpy(out, m->train_predictions.data(), m->train_predictions.size() * sizeof(double));
  });
}

}  // extern "C"

namespace {

// base + lr * sum of the given trees' leaves for every row, on the device.
void predict_trees(mpsb_cuda_backend* b, const std::vector<const std::vector<mpsb_tree_node>*>& trees,
                   double base, double lr, const mpsb_cuda_dataset* ds, double* out) {
  dataset_ready(ds);
  std::vector<uint32_t> offsets(trees.size() + 1, 0);
  for (size_t t = 0; t < trees.size(); ++t) {
    offsets[t + 1] = offsets[t] + uint32_t(trees[t]->size());
    for (const mpsb_tree_node& nd : *trees[t])
      if (!(nd.flags & 1u) && nd.feature_index >= ds->features)
        throw TrainingError("Prediction feature count does not match the tree model");
  }
  std::vector<mpsb_tree_node> flat(offsets.back() ? offsets.back() : 1);
  for (size_t t = 0; t < trees.size(); ++t)
    std::copy(trees[t]->begin(), trees[t]->end(), flat.begin() + offsets[t]);
  DevBuf d_nodes, d_off, d_out;
  d_nodes.alloc(flat.size() * sizeof(mpsb_tree_node));
  d_off.alloc(offsets.size() * sizeof(uint32_t));
  d_out.alloc(size_t(ds->n_rows) * sizeof(double));
  cudaStream_t s = b->stream;
  CK(cudaMemcpyAsync(d_nodes.p, flat.data(), flat.size() * sizeof(mpsb_tree_node), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d_off.p, offsets.data(), offsets.size() * 4, cudaMemcpyHostToDevice, s));
  CK(launch_predict(ds->bins_fm.as<uint8_t>(), ds->bins16_fm.as<uint16_t>(), ds->slots, ds->n_rows,
                    ds->nfb, ds->has_missing.as<uint8_t>(),
                    d_nodes.as<TreeNodeOut>(), d_off.as<uint32_t>(), uint32_t(trees.size()), base, lr,
                    d_out.as<double>(), b->error.as<uint32_t>(), s));
  CK(cudaMemcpyAsync(out, d_out.p, size_t(ds->n_rows) * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (b->take_error()) throw TrainingError("Tree node index is out of bounds or the structure contains a cycle");
}

}  // namespace

extern "C" {

int mpsb_cuda_model_predict(mpsb_cuda_backend* b, const mpsb_cuda_model* m,
                            const mpsb_cuda_dataset* ds, double* out) {
  return guard([&] {
    if (m->class_count) throw TrainingError("a softmax model predicts margins (mpsb_cuda_model_predict_margins)");
    b->activate();
    std::vector<const std::vector<mpsb_tree_node>*> trees;
    for (const auto& t : m->trees) trees.push_back(&t);
    predict_trees(b, trees, m->base, m->learning_rate, ds, out);
  });
}

int mpsb_cuda_model_predict_margins(mpsb_cuda_backend* b, const mpsb_cuda_model* m,
                                    const mpsb_cuda_dataset* ds, double* out) {
  return guard([&] {
    if (!m->class_count) throw TrainingError("not a softmax model");
    b->activate();
    const uint32_t K = m->class_count;
    std::vector<double> col(ds->n_rows);
    for (uint32_t k = 0; k < K; ++k) {  // class k owns trees k, k + K, ... (PredictMargins)
      std::vector<const std::vector<mpsb_tree_node>*> trees;
      for (size_t t = k; t < m->trees.size(); t += K) trees.push_back(&m->trees[t]);
      predict_trees(b, trees, m->base_scores[k], m->learning_rate, ds, col.data());
      for (uint32_t r = 0; r < ds->n_rows; ++r) out[size_t(r) * K + k] = col[r];
    }
  });
}

uint32_t mpsb_cuda_model_class_count(const mpsb_cuda_model* m) { return m->class_count; }

int mpsb_cuda_model_class_base_scores(const mpsb_cuda_model* m, double* out) {
  return guard([&] {
    if (!m->class_count) throw TrainingError("not a softmax model");
    std::copy(m->base_scores.begin(), m->base_scores.end(), out);
  });
}

int mpsb_cuda_model_class_labels(const mpsb_cuda_model* m, double* out) {
  return guard([&] {
    if (!m->class_count) throw TrainingError("not a softmax model");
    std::copy(m->class_labels.begin(), m->class_labels.end(), out);
  });
}

int mpsb_cuda_model_create_softmax(uint32_t class_count, double lr, const double* base_scores,
                                   const double* class_labels, uint32_t n_trees,
                                   const uint32_t* counts, const mpsb_tree_node* nodes,
                                   mpsb_cuda_model** out) {
  return guard([&] {
    if (class_count < 2 || n_trees == 0 || n_trees % class_count != 0 || !std::isfinite(lr) ||
        lr <= 0.0 || lr > 1.0)
      throw TrainingError("softmax model metadata is invalid");
    std::unique_ptr<mpsb_cuda_model> m(new mpsb_cuda_model);
    m->class_count = class_count;
    m->learning_rate = lr;
    m->base_scores.assign(base_scores, base_scores + class_count);
    for (double v : m->base_scores)
      if (!std::isfinite(v)) throw TrainingError("softmax model class metadata is not finite");
    m->class_labels.resize(class_count);
    for (uint32_t k = 0; k < class_count; ++k) {
      m->class_labels[k] = class_labels ? class_labels[k] : double(k);
      if (!std::isfinite(m->class_labels[k])) throw TrainingError("softmax model class metadata is not finite");
      if (k > 0 && !(m->class_labels[k - 1] < m->class_labels[k]))
        throw TrainingError("softmax model class labels must be strictly increasing");
    }
    m->n_trees = n_trees;
    m->trees.resize(n_trees);
    size_t off = 0;
    for (uint32_t t = 0; t < n_trees; ++t) {
      m->trees[t].assign(nodes + off, nodes + off + counts[t]);
      off += counts[t];
    }
    *out = m.release();
  });
}

void mpsb_cuda_model_destroy(mpsb_cuda_model* m) { delete m; }

}  // extern "C"
