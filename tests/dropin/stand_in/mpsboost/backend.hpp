// Stand-in for the reference's backend contract, so that the C++ adapter
// (include/mpsboost_cuda/cuda_backend.hpp) can be compiled and run on a machine that has a
// GPU but not the reference's sources. It declares, with the same names, members and
// signatures, exactly what the adapter uses from the reference's headers:
//   include/mpsboost/backend.hpp:22-25   BackendError
//   include/mpsboost/backend.hpp:40-47   HistogramBin, FeatureHistogram, NodeHistograms
//   include/mpsboost/backend.hpp:52-75   GradientComputer, HistogramBuilder
//   include/mpsboost/backend.hpp:124-135 LayerHistogramBuilder
//   include/mpsboost/objective.hpp:17-28 TrainingError, GradientPair
//   include/mpsboost/binned_dataset.hpp:18-110 DataError, BinStorage, FeatureBinMetadata and
//                                          the BinnedDataset accessors (feature-major u8 bins)
// The dataset here is a plain container the test fills; the reference's is built by
// QuantizeDense. Test infrastructure only.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace mpsboost {

class BackendError final : public std::runtime_error {
 public:
  explicit BackendError(const std::string& m) : std::runtime_error(m) {}
};
class TrainingError final : public std::runtime_error {
 public:
  explicit TrainingError(const std::string& m) : std::runtime_error(m) {}
};
class DataError final : public std::runtime_error {
 public:
  explicit DataError(const std::string& m) : std::runtime_error(m) {}
};

struct GradientPair final {
  double gradient{0.0};
  double hessian{0.0};
};

enum class BinStorage : std::uint8_t { kUInt8 = 1, kUInt16 = 2 };

struct FeatureBinMetadata final {
  std::uint64_t boundary_offset{0};
  std::uint32_t boundary_count{0};
  std::uint32_t bin_count{0};
  std::uint64_t missing_count{0};
};

class BinnedDataset {
 public:
  BinnedDataset(std::uint64_t rows, std::uint32_t features, std::vector<std::uint8_t> bins,
                std::vector<std::uint8_t> missing, std::vector<FeatureBinMetadata> metadata)
      : rows_(rows), features_(features), bins_(std::move(bins)), missing_(std::move(missing)),
        metadata_(std::move(metadata)) {}
  // u16 storage (max_bins above 256, binned_dataset.cpp:132).
  BinnedDataset(std::uint64_t rows, std::uint32_t features, std::vector<std::uint16_t> bins,
                std::vector<std::uint8_t> missing, std::vector<FeatureBinMetadata> metadata)
      : rows_(rows), features_(features), bins16_(std::move(bins)), missing_(std::move(missing)),
        metadata_(std::move(metadata)) {}
  std::uint64_t rows() const noexcept { return rows_; }
  std::uint32_t features() const noexcept { return features_; }
  BinStorage storage() const noexcept { return bins16_.empty() ? BinStorage::kUInt8 : BinStorage::kUInt16; }
  const std::vector<FeatureBinMetadata>& feature_metadata() const noexcept { return metadata_; }
  const void* bin_data() const noexcept {
    return bins16_.empty() ? static_cast<const void*>(bins_.data()) : static_cast<const void*>(bins16_.data());
  }
  bool IsMissing(std::uint64_t row, std::uint32_t feature) const {
    return missing_[static_cast<std::size_t>(feature) * rows_ + row] != 0;
  }
  std::uint32_t Bin(std::uint64_t row, std::uint32_t feature) const {
    const std::size_t i = static_cast<std::size_t>(feature) * rows_ + row;
    return bins16_.empty() ? bins_[i] : bins16_[i];
  }

 private:
  std::uint64_t rows_;
  std::uint32_t features_;
  std::vector<std::uint8_t> bins_;      // [features][rows], missing rows in bin 0
  std::vector<std::uint16_t> bins16_;   // the same, u16 storage
  std::vector<std::uint8_t> missing_;   // [features][rows]
  std::vector<FeatureBinMetadata> metadata_;
};

struct HistogramBin final {
  std::uint64_t count{0};
  double gradient_sum{0.0};
  double hessian_sum{0.0};
};
using FeatureHistogram = std::vector<HistogramBin>;
using NodeHistograms = std::vector<FeatureHistogram>;

class GradientComputer {
 public:
  virtual ~GradientComputer() = default;
  virtual std::vector<GradientPair> ComputeSquaredError(const std::vector<double>& labels,
                                                        const std::vector<double>& predictions) const = 0;
};

class HistogramBuilder {
 public:
  virtual ~HistogramBuilder() = default;
  virtual NodeHistograms BuildHistograms(const BinnedDataset& dataset, const std::vector<std::uint64_t>& rows,
                                         const std::vector<GradientPair>& gradients) const = 0;
};

class LayerHistogramBuilder {
 public:
  virtual ~LayerHistogramBuilder() = default;
  virtual std::vector<NodeHistograms> BuildLayerHistograms(
      const BinnedDataset& dataset, const std::vector<std::vector<std::uint64_t>>& node_rows,
      const std::vector<GradientPair>& gradients) const = 0;
};

}  // namespace mpsboost
