// C shim over the reference's own C++ core -- TEST INFRASTRUCTURE ONLY.
//
// Compiled together with the reference sources where they lie (oracle/Makefile); the
// result is oracle/_ref/libmpsb_ref.so. Its only purpose is to pin the plain-C
// restatement (oracle.c) and to generate golden fixtures. It calls only the
// reference's public API:
//   QuantizeDense / TransformDense        binned_dataset.hpp:137-144
//   ComputeSquaredErrorGradients & co.    objective.hpp:32-74
//   CpuReferenceBackend::BuildHistograms  backend.hpp:79-90
//   TrainSingleRegressionTree             tree.hpp:104-108
//   TrainRegressionModel                  trainer.hpp:133-139
//   TrainMulticlassSoftmaxModel           trainer.hpp:141-147
//   RegressionTree/RegressionModel::Predict
//   SerializeModel / DeserializeModel     trainer.hpp:152-153
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "mpsboost/backend.hpp"
#include "mpsboost/binned_dataset.hpp"
#include "mpsboost/objective.hpp"
#include "mpsboost/trainer.hpp"
#include "mpsboost/tree.hpp"

#include "oracle.h"

using namespace mpsboost;

namespace {

thread_local std::string g_error;

template <typename F>
int Guard(F&& body) {
  try {
    body();
    g_error.clear();
    return ORC_OK;
  } catch (const TrainingError& e) {
    g_error = e.what();
    return ORC_TRAINING_ERROR;
  } catch (const DataError& e) {
    g_error = e.what();
    return ORC_DATA_ERROR;
  } catch (const BackendError& e) {
    g_error = e.what();
    return ORC_BACKEND_ERROR;
  } catch (const std::exception& e) {
    g_error = e.what();
    return ORC_OTHER_ERROR;
  }
}

DenseMatrixView MakeView(const void* data, int scalar_type, std::uint64_t rows,
                         std::uint32_t features, std::uint64_t rs, std::uint64_t cs) {
  DenseMatrixView view;
  view.data = data;
  view.rows = rows;
  view.features = features;
  view.row_stride_bytes = rs;
  view.column_stride_bytes = cs;
  view.scalar_type = scalar_type == 2 ? ScalarType::kFloat64 : ScalarType::kFloat32;
  const std::uint64_t item = scalar_type == 2 ? 8 : 4;
  view.source_contiguous = (cs == item && rs == item * features);
  return view;
}

std::vector<GradientPair> Pairs(const double* pairs, std::uint64_t n) {
  std::vector<GradientPair> out(n);
  for (std::uint64_t i = 0; i < n; ++i) {
    out[i] = GradientPair{pairs[2 * i], pairs[2 * i + 1]};
  }
  return out;
}

TrainingParameters Params(const orc_params* p) {
  TrainingParameters t;
  t.n_estimators = p->n_estimators;
  t.learning_rate = p->learning_rate;
  t.max_bins = p->max_bins;
  t.objective = static_cast<TrainingParameters::Objective>(p->objective);
  t.objective_alpha = p->objective_alpha;
  t.tweedie_variance_power = p->tweedie_variance_power;
  TreeTrainingParameters& tree = t.tree;
  tree.max_depth = p->max_depth;
  tree.max_leaves = p->max_leaves;
  tree.max_active_leaves = p->max_active_leaves;
  tree.min_samples_leaf = p->min_samples_leaf;
  tree.min_child_weight = p->min_child_weight;
  tree.reg_lambda = p->reg_lambda;
  tree.reg_alpha = p->reg_alpha;
  tree.max_delta_step = p->max_delta_step;
  tree.gamma = p->gamma;
  tree.min_gain_to_split = p->min_gain_to_split;
  tree.split_strategy = static_cast<TreeTrainingParameters::SplitStrategy>(p->split_strategy);
  tree.growth_strategy = static_cast<TreeTrainingParameters::GrowthStrategy>(p->growth_strategy);
  tree.random_seed = p->random_seed;
  if (p->monotonic_constraints != nullptr) {
    tree.monotonic_constraints.assign(p->monotonic_constraints,
                                      p->monotonic_constraints + p->n_monotonic);
  }
  for (std::uint32_t g = 0; g < p->n_interaction_groups; ++g) {
    tree.interaction_constraints.emplace_back(
        p->interaction_features + p->interaction_offsets[g],
        p->interaction_features + p->interaction_offsets[g + 1]);
  }
  return t;
}

void CopyNodes(const RegressionTree& tree, orc_tree_node* out) {
  for (std::size_t i = 0; i < tree.nodes().size(); ++i) {
    const TreeNode& n = tree.nodes()[i];
    orc_tree_node o{};
    o.feature_index = n.feature_index;
    o.threshold_bin = n.threshold_bin;
    o.left_child = n.left_child;
    o.right_child = n.right_child;
    o.leaf_value = n.leaf_value;
    o.gain = n.gain;
    o.default_left = n.default_left ? 1 : 0;
    o.flags = n.flags;
    out[i] = o;
  }
}

const BinnedDataset& DS(const void* p) { return *static_cast<const BinnedDataset*>(p); }

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_error.c_str(); }

int ref_quantize_dense(const void* data, int scalar_type, std::uint64_t rows,
                       std::uint32_t features, std::uint64_t rs, std::uint64_t cs,
                       std::uint32_t max_bins, void** out) {
  return Guard([&] {
    *out = new BinnedDataset(
        QuantizeDense(MakeView(data, scalar_type, rows, features, rs, cs), max_bins));
  });
}

int ref_transform_dense(const void* schema_dataset, const void* data, int scalar_type,
                        std::uint64_t rows, std::uint32_t features, std::uint64_t rs,
                        std::uint64_t cs, void** out) {
  return Guard([&] {
    *out = new BinnedDataset(TransformDense(
        MakeView(data, scalar_type, rows, features, rs, cs), DS(schema_dataset).schema()));
  });
}

void ref_dataset_free(void* dataset) { delete static_cast<BinnedDataset*>(dataset); }

int ref_dataset_info(const void* dataset, std::uint64_t* rows, std::uint32_t* features,
                     std::uint32_t* max_bins, std::uint64_t* boundary_total) {
  return Guard([&] {
    *rows = DS(dataset).rows();
    *features = DS(dataset).features();
    *max_bins = DS(dataset).max_bins();
    *boundary_total = DS(dataset).boundaries().size();
  });
}

int ref_dataset_metadata(const void* dataset, std::uint64_t* boundary_offset,
                         std::uint32_t* boundary_count, std::uint32_t* bin_count,
                         std::uint64_t* missing_count) {
  return Guard([&] {
    const auto& meta = DS(dataset).feature_metadata();
    for (std::size_t f = 0; f < meta.size(); ++f) {
      boundary_offset[f] = meta[f].boundary_offset;
      boundary_count[f] = meta[f].boundary_count;
      bin_count[f] = meta[f].bin_count;
      missing_count[f] = meta[f].missing_count;
    }
  });
}

int ref_dataset_boundaries(const void* dataset, float* out) {
  return Guard([&] {
    const auto& b = DS(dataset).boundaries();
    std::memcpy(out, b.data(), b.size() * sizeof(float));
  });
}

int ref_dataset_bins(const void* dataset, std::uint16_t* out) {
  return Guard([&] {
    const BinnedDataset& ds = DS(dataset);
    for (std::uint32_t f = 0; f < ds.features(); ++f) {
      for (std::uint64_t r = 0; r < ds.rows(); ++r) {
        out[f * ds.rows() + r] = static_cast<std::uint16_t>(ds.GetBin(r, f));
      }
    }
  });
}

int ref_dataset_missing(const void* dataset, std::uint8_t* out) {
  return Guard([&] {
    const BinnedDataset& ds = DS(dataset);
    for (std::uint32_t f = 0; f < ds.features(); ++f) {
      for (std::uint64_t r = 0; r < ds.rows(); ++r) {
        out[f * ds.rows() + r] = ds.IsMissing(r, f) ? 1 : 0;
      }
    }
  });
}

int ref_gradients(std::uint32_t objective, double alpha, double variance_power,
                  const double* labels, const double* predictions, std::uint64_t n,
                  double* out_pairs) {
  return Guard([&] {
    const std::vector<double> y(labels, labels + n);
    const std::vector<double> p(predictions, predictions + n);
    std::vector<GradientPair> g;
    switch (objective) {
      case ORC_SQUARED_ERROR: g = ComputeSquaredErrorGradients(y, p); break;
      case ORC_BINARY_LOGISTIC: g = ComputeBinaryLogisticGradients(y, p); break;
      case ORC_QUANTILE: g = ComputeQuantileGradients(y, p, alpha); break;
      case ORC_POISSON: g = ComputePoissonGradients(y, p); break;
      case ORC_TWEEDIE: g = ComputeTweedieGradients(y, p, variance_power); break;
      default: throw TrainingError("unknown training objective");
    }
    for (std::uint64_t i = 0; i < n; ++i) {
      out_pairs[2 * i] = g[i].gradient;
      out_pairs[2 * i + 1] = g[i].hessian;
    }
  });
}

int ref_histograms(const void* dataset, const double* pairs, std::uint64_t n_pairs,
                   const std::uint64_t* rows, std::uint64_t n_rows, orc_hist_bin* out) {
  return Guard([&] {
    CpuReferenceBackend backend;
    const NodeHistograms h = backend.BuildHistograms(
        DS(dataset), std::vector<std::uint64_t>(rows, rows + n_rows), Pairs(pairs, n_pairs));
    std::size_t k = 0;
    for (const auto& feature : h) {
      for (const auto& bin : feature) {
        out[k++] = orc_hist_bin{bin.count, bin.gradient_sum, bin.hessian_sum};
      }
    }
  });
}

int ref_train_single_tree(const void* dataset, const double* pairs, std::uint64_t n,
                          const orc_params* params, void** tree_out) {
  return Guard([&] {
    CpuReferenceBackend backend;
    *tree_out = new RegressionTree(TrainSingleRegressionTree(
        DS(dataset), Pairs(pairs, n), Params(params).tree, backend));
  });
}

std::uint32_t ref_tree_node_count(const void* tree) {
  return static_cast<std::uint32_t>(static_cast<const RegressionTree*>(tree)->nodes().size());
}

int ref_tree_nodes(const void* tree, orc_tree_node* out) {
  return Guard([&] { CopyNodes(*static_cast<const RegressionTree*>(tree), out); });
}

int ref_tree_predict(const void* tree, const void* dataset, double* out) {
  return Guard([&] {
    const auto p = static_cast<const RegressionTree*>(tree)->Predict(DS(dataset));
    std::memcpy(out, p.data(), p.size() * sizeof(double));
  });
}

void ref_tree_free(void* tree) { delete static_cast<RegressionTree*>(tree); }

int ref_train_regressor(const void* dataset, const double* labels, const double* weights,
                        std::uint64_t n, const orc_params* params, void** model_out) {
  return Guard([&] {
    CpuReferenceBackend backend;
    *model_out = new RegressionModel(TrainRegressionModel(
        DS(dataset), std::vector<double>(labels, labels + n),
        std::vector<double>(weights, weights + n), Params(params), backend, backend));
  });
}

std::uint32_t ref_model_tree_count(const void* model) {
  return static_cast<const RegressionModel*>(model)->tree_count();
}

double ref_model_base_score(const void* model) {
  return static_cast<const RegressionModel*>(model)->base_score();
}

std::uint32_t ref_model_tree_node_count(const void* model, std::uint32_t tree) {
  return static_cast<std::uint32_t>(
      static_cast<const RegressionModel*>(model)->trees()[tree].nodes().size());
}

int ref_model_tree_nodes(const void* model, std::uint32_t tree, orc_tree_node* out) {
  return Guard([&] {
    CopyNodes(static_cast<const RegressionModel*>(model)->trees().at(tree), out);
  });
}

int ref_model_predict(const void* model, const void* dataset, double* out) {
  return Guard([&] {
    const auto p = static_cast<const RegressionModel*>(model)->Predict(DS(dataset));
    std::memcpy(out, p.data(), p.size() * sizeof(double));
  });
}

void ref_model_free(void* model) { delete static_cast<RegressionModel*>(model); }

int ref_train_softmax(const void* dataset, const double* labels, const double* weights,
                      std::uint64_t n, const orc_params* params, std::uint32_t class_count,
                      void** model_out) {
  return Guard([&] {
    CpuReferenceBackend backend;
    *model_out = new MulticlassModel(TrainMulticlassSoftmaxModel(
        DS(dataset), std::vector<double>(labels, labels + n),
        std::vector<double>(weights, weights + n), Params(params), class_count, backend));
  });
}

std::uint32_t ref_softmax_tree_count(const void* model) {
  return static_cast<const MulticlassModel*>(model)->tree_count();
}

std::uint32_t ref_softmax_class_count(const void* model) {
  return static_cast<const MulticlassModel*>(model)->class_count();
}

int ref_softmax_base_scores(const void* model, double* out) {
  return Guard([&] {
    const auto& b = static_cast<const MulticlassModel*>(model)->base_scores();
    std::memcpy(out, b.data(), b.size() * sizeof(double));
  });
}

std::uint32_t ref_softmax_tree_node_count(const void* model, std::uint32_t tree) {
  return static_cast<std::uint32_t>(
      static_cast<const MulticlassModel*>(model)->trees()[tree].nodes().size());
}

int ref_softmax_tree_nodes(const void* model, std::uint32_t tree, orc_tree_node* out) {
  return Guard([&] {
    CopyNodes(static_cast<const MulticlassModel*>(model)->trees().at(tree), out);
  });
}

int ref_softmax_predict_margins(const void* model, const void* dataset, double* out) {
  return Guard([&] {
    const auto p = static_cast<const MulticlassModel*>(model)->PredictMargins(DS(dataset));
    std::memcpy(out, p.data(), p.size() * sizeof(double));
  });
}

void ref_softmax_free(void* model) { delete static_cast<MulticlassModel*>(model); }

int ref_model_serialize(const void* model, std::uint8_t* out, std::uint64_t capacity,
                        std::uint64_t* size) {
  return Guard([&] {
    const std::vector<std::uint8_t> bytes = SerializeModel(*static_cast<const RegressionModel*>(model));
    *size = bytes.size();
    if (out != nullptr && capacity >= bytes.size()) std::memcpy(out, bytes.data(), bytes.size());
  });
}

int ref_softmax_serialize(const void* model, std::uint8_t* out, std::uint64_t capacity,
                          std::uint64_t* size) {
  return Guard([&] {
    const std::vector<std::uint8_t> bytes = SerializeModel(*static_cast<const MulticlassModel*>(model));
    *size = bytes.size();
    if (out != nullptr && capacity >= bytes.size()) std::memcpy(out, bytes.data(), bytes.size());
  });
}

int ref_softmax_deserialize(const std::uint8_t* data, std::uint64_t size, void** model_out) {
  return Guard([&] {
    *model_out = new MulticlassModel(DeserializeMulticlassModel(std::vector<std::uint8_t>(data, data + size)));
  });
}

int ref_model_deserialize(const std::uint8_t* data, std::uint64_t size, void** model_out) {
  return Guard([&] {
    *model_out = new RegressionModel(DeserializeModel(std::vector<std::uint8_t>(data, data + size)));
  });
}

}  // extern "C"
