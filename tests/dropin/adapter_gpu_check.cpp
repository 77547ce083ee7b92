// The C++ adapter (include/mpsboost_cuda/cuda_backend.hpp) driven through the backend
// contract on a GPU, compiled against the stand-in declarations in stand_in/: capability
// detection by dynamic_cast (as tree_histogram.cpp:83-84 does), squared-error gradients,
// layer and node histograms against FP64 row-order sums on the host (count exact, G within
// 2e-5 and H within 1e-6, the reference's GPU tolerances, tests/metal/test_mps_histogram.py),
// missing rows in bin 0, a second dataset replacing the resident one, a u16 dataset (up to
// 4000 bins), and the contract's errors. Prints "adapter ok" on success; exits non-zero with a message otherwise.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "mpsboost/backend.hpp"
#include "mpsboost_cuda/cuda_backend.hpp"

using namespace mpsboost;

static int fail(const char* what) {
  std::printf("FAIL: %s\n", what);
  return 1;
}

// u8 storage with 2 .. 255 bins per feature, or (wide) u16 storage with up to 4000 bins.
static BinnedDataset make_dataset(std::uint64_t rows, std::uint32_t features, unsigned seed,
                                  bool wide = false) {
  std::mt19937_64 gen(seed);
  std::vector<std::uint16_t> bins(rows * features);
  std::vector<std::uint8_t> missing(rows * features, 0);
  std::vector<FeatureBinMetadata> meta(features);
  for (std::uint32_t f = 0; f < features; ++f) {
    meta[f].bin_count = wide ? 2 + (f * 997) % 3999 : 2 + (f * 37) % 254;
    for (std::uint64_t r = 0; r < rows; ++r) {
      const std::size_t c = std::size_t(f) * rows + r;
      if (f % 3 == 0 && gen() % 10 == 0) {  // every third feature has missing values
        missing[c] = 1;
        bins[c] = 0;
        ++meta[f].missing_count;
      } else {
        bins[c] = std::uint16_t(gen() % meta[f].bin_count);
      }
    }
  }
  if (wide) return BinnedDataset(rows, features, std::move(bins), std::move(missing), std::move(meta));
  return BinnedDataset(rows, features, std::vector<std::uint8_t>(bins.begin(), bins.end()), std::move(missing),
                       std::move(meta));
}

static bool check_node(const BinnedDataset& ds, const std::vector<std::uint64_t>& rows,
                       const std::vector<GradientPair>& gp, const NodeHistograms& got) {
  if (got.size() != ds.features()) return false;
  for (std::uint32_t f = 0; f < ds.features(); ++f) {
    FeatureHistogram want(ds.feature_metadata()[f].bin_count);
    for (std::uint64_t r : rows) {  // missing rows are counted in bin 0
      HistogramBin& b = want[ds.IsMissing(r, f) ? 0 : ds.Bin(r, f)];
      ++b.count;
      b.gradient_sum += gp[r].gradient;
      b.hessian_sum += gp[r].hessian;
    }
    if (got[f].size() != want.size()) return false;
    for (std::size_t k = 0; k < want.size(); ++k) {
      if (got[f][k].count != want[k].count) return false;
      if (std::fabs(got[f][k].gradient_sum - want[k].gradient_sum) > 2e-5 * std::max(1.0, std::fabs(want[k].gradient_sum)))
        return false;
      if (std::fabs(got[f][k].hessian_sum - want[k].hessian_sum) > 1e-6 * std::max(1.0, std::fabs(want[k].hessian_sum)))
        return false;
    }
  }
  return true;
}

int main() {
  CudaBackend backend(0);
  const HistogramBuilder& builder = backend;
  if (dynamic_cast<const LayerHistogramBuilder*>(&builder) == nullptr) return fail("layer capability not detected");

  const std::uint64_t n = 50000;
  std::vector<double> labels(n), preds(n);
  std::mt19937_64 gen(11);
  std::normal_distribution<double> normal(0.0, 1.0);
  for (std::uint64_t i = 0; i < n; ++i) {
    labels[i] = normal(gen);
    preds[i] = 0.25 * normal(gen);
  }
  const std::vector<GradientPair> gp = backend.ComputeSquaredError(labels, preds);
  for (std::uint64_t i = 0; i < n; ++i)
    if (gp[i].gradient != preds[i] - labels[i] || gp[i].hessian != 1.0) return fail("squared-error gradients");
  std::vector<GradientPair> weighted(gp);
  for (std::uint64_t i = 0; i < n; ++i) weighted[i].hessian = 0.5 + double(i % 7) / 7.0;

  // The second dataset replaces the resident one; the third stores u16 bins.
  for (unsigned round = 0; round < 3; ++round) {
    const BinnedDataset ds = make_dataset(n, round == 0 ? 70 : (round == 1 ? 33 : 9), 100 + round, round == 2);
    std::vector<std::vector<std::uint64_t>> nodes(3);
    for (std::uint64_t r = 0; r < n; ++r) nodes[(r * 2654435761u >> 7) % 3].push_back(r);
    nodes[2].resize(nodes[2].size() / 4);  // a small node
    const std::vector<NodeHistograms> layer = backend.BuildLayerHistograms(ds, nodes, weighted);
    if (layer.size() != nodes.size()) return fail("layer size");
    for (std::size_t i = 0; i < nodes.size(); ++i)
      if (!check_node(ds, nodes[i], weighted, layer[i])) return fail("layer histogram against FP64 sums");
    const NodeHistograms single = backend.BuildHistograms(ds, nodes[1], weighted);  // resident dataset
    for (std::uint32_t f = 0; f < ds.features(); ++f)
      for (std::size_t k = 0; k < single[f].size(); ++k)
        if (single[f][k].count != layer[1][f][k].count || single[f][k].gradient_sum != layer[1][f][k].gradient_sum ||
            single[f][k].hessian_sum != layer[1][f][k].hessian_sum)
          return fail("node histogram differs from the same node in a layer");
  }

  bool threw = false;
  try {
    backend.ComputeSquaredError({}, {});
  } catch (const TrainingError&) {
    threw = true;
  }
  if (!threw) return fail("empty labels accepted");
  threw = false;
  try {
    backend.ComputeSquaredError({1.0, 2.0}, {1.0});
  } catch (const TrainingError&) {
    threw = true;
  }
  if (!threw) return fail("mismatched lengths accepted");
  std::printf("adapter ok\n");
  return 0;
}
