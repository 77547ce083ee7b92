// CudaBackend: the GB300 CUDA backend as a drop-in for MPSBoost's C++ backend contract.
//
// Header-only adapter over the C ABI (mpsb_cuda.h) for a build of the reference core: it
// derives from the reference's own interfaces in include/mpsboost/backend.hpp --
// GradientComputer (52-58), HistogramBuilder (64-75) and LayerHistogramBuilder (124-135) --
// exactly as MpsBackend does (140-195), so TrainRegressionModel / TrainSingleRegressionTree
// take it unchanged and detect the layer capability with the same dynamic_cast
// (src/core/tree_histogram.cpp:83-84, 122-123).
//
// The binned matrix is uploaded once per dataset and kept resident (MpsBackend re-uploads
// it for every node, src/mps/mps_histogram.mm:149). Like MpsBackend it keeps mutable
// device state, so use one backend per thread. Errors raise the reference's exception
// types: TrainingError for contract violations, BackendError for device failures.
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mpsboost/backend.hpp"
#include "mpsb_cuda.h"

namespace mpsboost {

class CudaBackend final : public GradientComputer,
                          public HistogramBuilder,
                          public LayerHistogramBuilder {
 public:
  explicit CudaBackend(int device = 0, int hist_mode = MPSB_HIST_FIXED) {
    Check(mpsb_cuda_backend_create(device, &backend_), "CUDA backend creation");
    Check(mpsb_cuda_backend_set_hist_mode(backend_, hist_mode), "histogram mode");
  }
  ~CudaBackend() override {
    if (dataset_) mpsb_cuda_dataset_destroy(dataset_);
    if (backend_) mpsb_cuda_backend_destroy(backend_);
  }
  CudaBackend(CudaBackend&& other) noexcept { *this = std::move(other); }
  CudaBackend& operator=(CudaBackend&& other) noexcept {
    std::swap(backend_, other.backend_);
    std::swap(dataset_, other.dataset_);
    std::swap(key_, other.key_);
    return *this;
  }
  CudaBackend(const CudaBackend&) = delete;
  CudaBackend& operator=(const CudaBackend&) = delete;

  std::vector<GradientPair> ComputeSquaredError(
      const std::vector<double>& labels,
      const std::vector<double>& predictions) const override {
    if (labels.empty()) throw TrainingError("Labels must not be empty");
    if (labels.size() != predictions.size())
      throw TrainingError("Label and prediction lengths do not match");
    std::vector<double> pairs(2 * labels.size());
    Check(mpsb_cuda_squared_error(backend_, labels.data(), predictions.data(), labels.size(),
                                  pairs.data()),
          "squared-error gradients");
    std::vector<GradientPair> out(labels.size());
    for (std::size_t i = 0; i < out.size(); ++i) out[i] = GradientPair{pairs[2 * i], pairs[2 * i + 1]};
    return out;
  }

  NodeHistograms BuildHistograms(const BinnedDataset& dataset,
                                 const std::vector<std::uint64_t>& rows,
                                 const std::vector<GradientPair>& gradients) const override {
    return BuildLayerHistograms(dataset, {rows}, gradients).front();
  }

  std::vector<NodeHistograms> BuildLayerHistograms(
      const BinnedDataset& dataset,
      const std::vector<std::vector<std::uint64_t>>& node_rows,
      const std::vector<GradientPair>& gradients) const override {
    if (node_rows.empty()) return {};
    mpsb_cuda_dataset* ds = Resident(dataset);
    std::vector<std::uint64_t> rows, offsets{0};
    for (const auto& node : node_rows) {
      rows.insert(rows.end(), node.begin(), node.end());
      offsets.push_back(rows.size());
    }
    std::vector<double> pairs(2 * gradients.size());
    for (std::size_t i = 0; i < gradients.size(); ++i) {
      pairs[2 * i] = gradients[i].gradient;
      pairs[2 * i + 1] = gradients[i].hessian;
    }
    std::size_t per_node = 0;
    for (const auto& m : dataset.feature_metadata()) per_node += m.bin_count;
    std::vector<mpsb_histogram_bin> flat(per_node * node_rows.size());
    Check(mpsb_cuda_build_layer_histograms(backend_, ds, rows.data(), offsets.data(),
                                           static_cast<std::uint32_t>(node_rows.size()),
                                           pairs.data(), gradients.size(), flat.data()),
          "layer histograms");
    std::vector<NodeHistograms> out(node_rows.size());
    std::size_t k = 0;
    for (auto& node : out) {
      node.reserve(dataset.features());
      for (const auto& m : dataset.feature_metadata()) {
        FeatureHistogram feature(m.bin_count);
        for (auto& bin : feature) {
          bin = HistogramBin{flat[k].count, flat[k].gradient_sum, flat[k].hessian_sum};
          ++k;
        }
        node.push_back(std::move(feature));
      }
    }
    return out;
  }

 private:
  // Upload the dataset once; later calls with the same dataset reuse the device copy.
  mpsb_cuda_dataset* Resident(const BinnedDataset& dataset) const {
    const Key key{dataset.bin_data(), dataset.rows(), dataset.features()};
    if (dataset_ && key.data == key_.data && key.rows == key_.rows && key.features == key_.features)
      return dataset_;
    if (dataset_) mpsb_cuda_dataset_destroy(dataset_);
    dataset_ = nullptr;
    const std::uint32_t features = dataset.features();
    std::vector<std::uint32_t> bin_count(features);
    std::vector<std::uint8_t> missing;
    for (std::uint32_t f = 0; f < features; ++f) {
      const FeatureBinMetadata& m = dataset.feature_metadata()[f];
      bin_count[f] = m.bin_count;
      if (m.missing_count == 0) continue;
      if (missing.empty()) missing.assign(static_cast<std::size_t>(dataset.rows()) * features, 0);
      for (std::uint64_t r = 0; r < dataset.rows(); ++r)
        missing[f * dataset.rows() + r] = dataset.IsMissing(r, f) ? 1 : 0;
    }
    const std::uint32_t width = dataset.storage() == BinStorage::kUInt8 ? 1 : 2;
    Check(mpsb_cuda_dataset_create(backend_, dataset.bin_data(), width,
                                   missing.empty() ? nullptr : missing.data(), dataset.rows(),
                                   features, bin_count.data(), &dataset_),
          "dataset upload");
    key_ = key;
    return dataset_;
  }

  static void Check(int rc, const char* stage) {
    if (rc == MPSB_OK) return;
    const std::string msg = std::string(stage) + ": " + mpsb_cuda_last_error();
    if (rc == MPSB_ERR_TRAINING) throw TrainingError(msg);
    if (rc == MPSB_ERR_DATA) throw DataError(msg);
    throw BackendError(msg);
  }

  struct Key {
    const void* data;
    std::uint64_t rows;
    std::uint32_t features;
  };
  mpsb_cuda_backend* backend_ = nullptr;
  mutable mpsb_cuda_dataset* dataset_ = nullptr;
  mutable Key key_{nullptr, 0, 0};
};

}  // namespace mpsboost
