// Private host-side types of the CUDA backend (shared by host.cu and node_entries.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/mpsb_cuda.h"
#include "host_errors.h"
#include "kernels.h"

namespace mpsb {

extern thread_local std::string g_error;

// Allocator whose resize() leaves new elements uninitialized: buffers that a device copy
// fills right away skip the zero fill (and its first-touch page faults).
template <class T>
struct NoInitAllocator : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInitAllocator<U>;
  };
  NoInitAllocator() = default;
  template <class U>
  NoInitAllocator(const NoInitAllocator<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <class U, class... Args>
  void construct(U* p, Args&&... args) {
    ::new (static_cast<void*>(p)) U(std::forward<Args>(args)...);
  }
};

template <class F>
int guard(F&& body) {
  try {
    body();
    g_error.clear();
    return MPSB_OK;
  } catch (const Error& e) {
    g_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_error = "out of host memory";
    return MPSB_ERR_BACKEND;
  } catch (const std::exception& e) {
    g_error = e.what();
    return MPSB_ERR_BACKEND;
  }
}

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw BackendError(std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(expr) ::mpsb::cuda_check((expr), #expr)

// Owning device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void alloc(size_t n) {
    reset();
    if (n == 0) n = 16;
    const cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      throw BackendError("cudaMalloc of " + std::to_string(n) + " bytes failed: " +
                         cudaGetErrorString(e));
    }
    bytes = n;
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

std::string describe_device_error(uint32_t bits);
void attach_bins_tmap(mpsb_cuda_dataset* d);
void fixed_scales(const float* pairs32, uint64_t n, uint64_t n_rows, int32_t* kg, int32_t* kh);
void validate_tree_params(const mpsb_train_params& p, uint32_t features);
// Histogram slots per feature for these bin counts and missing flags: 256 when every
// feature's bins and missing slot fit in 256, else the next multiple of 256 (at most 65536;
// a feature with missing values then has at most 65535 bins).
uint32_t dataset_slots(const uint32_t* bin_count, const uint8_t* has_missing, uint32_t features);

}  // namespace mpsb

struct mpsb_cuda_backend {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host-to-device uploads that overlap kernels
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  int hist_mode = MPSB_HIST_FIXED;
  int sm_count = 0;
  cudaDeviceProp prop{};
  mpsb::DevBuf error;  // one uint32 status word for standalone kernels

  void activate() const { CK(cudaSetDevice(device)); }
  uint32_t take_error() {
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, error.p, sizeof e, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (e) CK(cudaMemsetAsync(error.p, 0, sizeof(uint32_t), stream));
    return e;
  }
  ~mpsb_cuda_backend() {
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (stream) cudaStreamDestroy(stream);
  }
};

struct mpsb_cuda_dataset {
  mpsb_cuda_backend* backend = nullptr;
  uint32_t n_rows = 0, features = 0, nfb = 0;
  // Histogram slots per feature: 256 (u8 copies bins, bins_blocked, bins_fm; missing rows
  // at 255) or, for a wide dataset, the multiple of 256 that holds every feature's bins and
  // its missing slot (u16 copies bins16, bins16_fm; missing rows at slots - 1).
  uint32_t slots = 256;
  mpsb::DevBuf bins, bins_blocked, bins_fm, bin_count, has_missing;
  mpsb::DevBuf bins16, bins16_fm;
  CUtensorMap bins_tmap{};  // row-major bins for TMA gathers (valid when has_bins_tmap)
  bool has_bins_tmap = false;
  std::vector<uint32_t> h_bin_count;
  std::vector<uint8_t> h_has_missing;
  // Quantization schema (datasets binned on the device): boundaries per feature.
  bool has_schema = false;
  uint32_t max_bins = 0;
  std::vector<float> boundaries;
  std::vector<uint64_t> boundary_offset;
  std::vector<uint32_t> boundary_count;
  std::vector<uint64_t> missing_count;
  // Upload state. An asynchronous upload (mpsb_cuda_dataset_create_async) is pending until
  // mpsb::dataset_ready has waited for `ready`: until then the staging buffers stay alive
  // and the pack kernels' range error (`pack_error`) is unread. Work on the backend's
  // stream is ordered after the packs, so only the host needs to wait.
  mutable std::mutex ready_mutex;  // threads sharing a pending dataset complete it once
  mutable bool pending = false;
  mutable bool invalid = false;
  cudaEvent_t ready = nullptr;
  mpsb::DevBuf pack_error;
  mutable mpsb::DevBuf stage[2], mstage[2];
  mpsb_cuda_dataset() = default;
  mpsb_cuda_dataset(const mpsb_cuda_dataset&) = delete;
  mpsb_cuda_dataset& operator=(const mpsb_cuda_dataset&) = delete;
  ~mpsb_cuda_dataset() {
    if (ready) {
      cudaEventSynchronize(ready);  // copies in flight read the staging buffers
      cudaEventDestroy(ready);
    }
  }
};

namespace mpsb {
// Completes a pending upload: waits for the packs, releases the staging buffers and throws
// DataError for a bin past its feature's count. Every entry that reads a dataset's device
// arrays calls it first; it returns at once for a complete upload.
void dataset_ready(const mpsb_cuda_dataset* d);
}  // namespace mpsb

struct mpsb_cuda_model {
  uint32_t n_trees = 0;
  double base = 0.0, learning_rate = 0.1;
  std::vector<std::vector<mpsb_tree_node>> trees;
  std::vector<double, mpsb::NoInitAllocator<double>> train_predictions;  // softmax margins
  // Training predictions of a trained regression model stay on the device (a copy of the
  // trainer's) until a caller asks for them.
  mpsb::DevBuf device_predictions;
  uint64_t device_prediction_count = 0;
  int device = 0;
  // Native softmax models: class count (0 for regression), per-class base scores and
  // class labels; trees are ordered (round, class).
  uint32_t class_count = 0;
  std::vector<double> base_scores, class_labels;
  // Objective metadata and the training data's quantization schema (the model file's).
  uint32_t objective = 0;
  double objective_alpha = 0.5, tweedie_variance_power = 1.5;
  bool has_schema = false;
  uint32_t features = 0, max_bins = 0;
  std::vector<float> boundaries;
  std::vector<uint64_t> boundary_offset, missing_count;
  std::vector<uint32_t> boundary_count, bin_count;
};

