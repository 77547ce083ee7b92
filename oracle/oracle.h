/*
 * CPU oracle for the MPSBoost GBDT training hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Two libraries export this same API under two prefixes:
 *   orc_*  : oracle/oracle.c, a plain-C restatement of the reference algorithm
 *            (quantization, objectives, FP64 row-ordered histograms, split scan,
 *            partition, level-wise tree growth, boosting loop, prediction), plus a
 *            CPU fixed-point replica of the int64 histogram path of the CUDA backend.
 *   ref_*  : oracle/ref_shim.cpp linked against the reference's own C++ core,
 *            compiled in place from its sources (see oracle/Makefile). It only
 *            exists where the reference sources exist and is used to pin orc_*.
 *
 * Only tests, the smoke check and the benchmark's CPU-baseline leg may load either
 * library. Nothing in the product links or calls it.
 *
 * Reference files followed (paths inside the reference project):
 *   include/mpsboost/backend.hpp:40-47 (HistogramBin)      -> orc_hist_bin
 *   include/mpsboost/tree.hpp:31-72 (TreeNode, parameters) -> orc_tree_node, orc_params
 *   include/mpsboost/trainer.hpp:20-36 (TrainingParameters)-> orc_params
 */
#ifndef MPSB_ORACLE_H
#define MPSB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Objective ids follow TrainingParameters::Objective (trainer.hpp:21-27). */
enum { ORC_SQUARED_ERROR = 0, ORC_BINARY_LOGISTIC = 1, ORC_QUANTILE = 2,
       ORC_POISSON = 3, ORC_TWEEDIE = 4 };
/* Histogram arithmetic used while growing trees (orc_* only). */
enum { ORC_HIST_FP64 = 0,   /* reference: FP64 gradients, row-ordered FP64 sums */
       ORC_HIST_FIXED = 1 }; /* replica: FP32 g/h -> scaled int64, exact sums     */

/* Error codes: 0 ok; 1 TrainingError; 2 DataError; 3 BackendError; 4 other. */
enum { ORC_OK = 0, ORC_TRAINING_ERROR = 1, ORC_DATA_ERROR = 2,
       ORC_BACKEND_ERROR = 3, ORC_OTHER_ERROR = 4 };

typedef struct {
  uint32_t n_estimators;
  uint32_t max_bins;
  uint32_t objective;
  uint32_t max_depth;
  uint32_t max_leaves;
  uint32_t max_active_leaves;
  uint32_t split_strategy;   /* 0 best_gain, 1 random_threshold */
  uint32_t growth_strategy;  /* 0 level_wise, 1 leaf_wise */
  uint32_t random_seed;
  uint32_t n_monotonic;
  uint32_t n_interaction_groups;
  uint32_t reserved;
  uint64_t min_samples_leaf;
  double learning_rate;
  double objective_alpha;
  double tweedie_variance_power;
  double min_child_weight;
  double reg_lambda;
  double reg_alpha;
  double max_delta_step;
  double gamma;
  double min_gain_to_split;
  const int8_t* monotonic_constraints;   /* n_monotonic entries or NULL */
  const uint32_t* interaction_offsets;   /* n_interaction_groups + 1 entries */
  const uint32_t* interaction_features;  /* concatenated groups */
} orc_params;

typedef struct {
  uint32_t feature_index;
  uint32_t threshold_bin;
  uint32_t left_child;
  uint32_t right_child;
  double leaf_value;
  double gain;
  uint8_t default_left;
  uint8_t flags;
  uint8_t reserved[6];
} orc_tree_node;

typedef struct {
  uint64_t count;
  double gradient_sum;
  double hessian_sum;
} orc_hist_bin;

/* Fixed-point bin of the replica: exact integer sums of quantized FP32 g/h. */
typedef struct {
  uint64_t count;
  int64_t gradient_q;
  int64_t hessian_q;
} orc_fixed_bin;

#define ORC_DECLARE_API(P)                                                           \
  const char* P##last_error(void);                                                   \
  int P##quantize_dense(const void* data, int scalar_type, uint64_t rows,            \
                        uint32_t features, uint64_t row_stride_bytes,                \
                        uint64_t column_stride_bytes, uint32_t max_bins,             \
                        void** out);                                                 \
  int P##transform_dense(const void* schema_dataset, const void* data,               \
                         int scalar_type, uint64_t rows, uint32_t features,          \
                         uint64_t row_stride_bytes, uint64_t column_stride_bytes,    \
                         void** out);                                                \
  void P##dataset_free(void* dataset);                                               \
  int P##dataset_info(const void* dataset, uint64_t* rows, uint32_t* features,       \
                      uint32_t* max_bins, uint64_t* boundary_total);                 \
  int P##dataset_metadata(const void* dataset, uint64_t* boundary_offset,            \
                          uint32_t* boundary_count, uint32_t* bin_count,             \
                          uint64_t* missing_count);                                  \
  int P##dataset_boundaries(const void* dataset, float* out);                        \
  int P##dataset_bins(const void* dataset, uint16_t* out);                           \
  int P##dataset_missing(const void* dataset, uint8_t* out);                         \
  int P##gradients(uint32_t objective, double alpha, double variance_power,          \
                   const double* labels, const double* predictions, uint64_t n,      \
                   double* out_pairs);                                               \
  int P##histograms(const void* dataset, const double* pairs, uint64_t n_pairs,      \
                    const uint64_t* rows, uint64_t n_rows, orc_hist_bin* out);       \
  int P##train_single_tree(const void* dataset, const double* pairs, uint64_t n,     \
                           const orc_params* params, void** tree_out);               \
  uint32_t P##tree_node_count(const void* tree);                                     \
  int P##tree_nodes(const void* tree, orc_tree_node* out);                           \
  int P##tree_predict(const void* tree, const void* dataset, double* out);           \
  void P##tree_free(void* tree);                                                     \
  int P##train_regressor(const void* dataset, const double* labels,                  \
                         const double* weights, uint64_t n,                          \
                         const orc_params* params, void** model_out);                \
  uint32_t P##model_tree_count(const void* model);                                   \
  double P##model_base_score(const void* model);                                     \
  uint32_t P##model_tree_node_count(const void* model, uint32_t tree);               \
  int P##model_tree_nodes(const void* model, uint32_t tree, orc_tree_node* out);     \
  int P##model_predict(const void* model, const void* dataset, double* out);         \
  void P##model_free(void* model);                                                   \
  /* TrainMulticlassSoftmaxModel (trainer.hpp:141-147) and MulticlassModel */          \
  int P##train_softmax(const void* dataset, const double* labels,                    \
                       const double* weights, uint64_t n, const orc_params* params,  \
                       uint32_t class_count, void** model_out);                      \
  uint32_t P##softmax_tree_count(const void* model);                                 \
  uint32_t P##softmax_class_count(const void* model);                                \
  int P##softmax_base_scores(const void* model, double* out);                        \
  uint32_t P##softmax_tree_node_count(const void* model, uint32_t tree);             \
  int P##softmax_tree_nodes(const void* model, uint32_t tree, orc_tree_node* out);   \
  int P##softmax_predict_margins(const void* model, const void* dataset, double* out); \
  void P##softmax_free(void* model);

ORC_DECLARE_API(orc_)
ORC_DECLARE_API(ref_)

/* ---- ref_* only: the reference's model file codec (SerializeModel / DeserializeModel,
   trainer.hpp:152-153), used to pin the library's model files ---- */
int ref_model_serialize(const void* model, uint8_t* out, uint64_t capacity, uint64_t* size);
int ref_model_deserialize(const uint8_t* data, uint64_t size, void** model_out);
int ref_softmax_serialize(const void* model, uint8_t* out, uint64_t capacity, uint64_t* size);
int ref_softmax_deserialize(const uint8_t* data, uint64_t size, void** model_out);

/* ---- orc_* only: the fixed-point replica and finer-grained hooks ---- */

/* Power-of-two scale exponents of one round: q_g = rne(g * 2^kg), q_h = rne(h * 2^kh). */
int orc_fixed_scales(const float* pairs32, uint64_t n, int32_t* kg, int32_t* kh);
/* Port only: threads of the feature-parallel loops (0 = all cores). Results do not
   depend on it. */
void orc_set_threads(int threads);
/* Exact int64 histograms of FP32 pairs. Output: features x bin_count bins (bin 0 holds
   the non-missing rows of bin 0 only) followed by one missing-statistics bin per feature. */
int orc_fixed_histograms(const void* dataset, const float* pairs32, int32_t kg,
                         int32_t kh, const uint64_t* rows, uint64_t n_rows,
                         orc_fixed_bin* out_bins, orc_fixed_bin* out_missing);
int orc_train_single_tree_fixed(const void* dataset, const float* pairs32, uint64_t n,
                                int32_t kg, int32_t kh, const orc_params* params,
                                void** tree_out);
int orc_train_softmax_mode(const void* dataset, const double* labels, const double* weights,
                           uint64_t n, const orc_params* params, uint32_t class_count,
                           int hist_mode, void** model_out);
int orc_train_regressor_mode(const void* dataset, const double* labels,
                             const double* weights, uint64_t n, const orc_params* params,
                             int hist_mode, void** model_out);
/* Per-feature best split of one node (full FindBestSplit semantics per feature), the
   shape of MpsBackend::ScanSplitsForTest (backend.hpp:173-180). */
typedef struct {
  uint32_t valid;
  uint32_t feature;
  uint32_t threshold_bin;
  uint32_t default_left;
  uint64_t left_count;
  uint64_t right_count;
  double left_gradient_sum;
  double left_hessian_sum;
  double right_gradient_sum;
  double right_hessian_sum;
  double gain;
} orc_split_candidate;
int orc_scan_splits(const void* dataset, const double* pairs, uint64_t n,
                    const uint64_t* rows, uint64_t n_rows, const orc_params* params,
                    orc_split_candidate* out_per_feature);
/* Stable partition of node rows, the rule of tree_split.cpp:273-285. */
int orc_partition_rows(const void* dataset, const uint64_t* rows, uint64_t n_rows,
                       uint32_t feature, uint32_t threshold_bin, int default_left,
                       uint64_t* left_out, uint64_t* right_out, uint64_t* n_left);
/* The materialized sample of a forest tree, matrix[rows][:, features] with the source's
   bins and boundaries (rows may repeat; features in the given order). Missing counts are
   recomputed for the sample. The schema of _ForestMixin's per-tree fit
   (forest_sampling.py:56-60) when the sample keeps the full data's bin boundaries. */
int orc_dataset_subset(const void* dataset, const uint64_t* rows, uint64_t n_rows,
                       const uint32_t* features, uint32_t n_features, void** out);
/* A dataset from feature-major bins (u8 or u16) and a missing mask computed elsewhere
   under the given schema; missing cells hold bin 0, as QuantizeDense leaves them. */
int orc_dataset_from_bins(const void* bins, uint32_t width, const uint8_t* missing,
                          uint64_t rows, uint32_t features, uint32_t max_bins,
                          const float* boundaries, const uint64_t* boundary_offset,
                          const uint32_t* boundary_count, const uint32_t* bin_count, void** out);
/* Weighted FP64 gradients of one boosting round rounded to FP32, the input of the
   fixed-point replica (trainer.cpp:178-216 followed by a round-to-nearest cast). */
int orc_weighted_pairs32(uint32_t objective, double alpha, double variance_power,
                         const double* labels, const double* predictions,
                         const double* weights, uint64_t n, float* out_pairs32);

#ifdef __cplusplus
}
#endif

#endif
