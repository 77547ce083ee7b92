/*
 * mpsb_cuda.h -- C ABI of the GB300 (sm_103a) CUDA backend for the MPSBoost GBDT
 * training hot path: gradient/hessian -> histogram build (+ sibling subtraction) ->
 * split-gain scan -> row partition.
 *
 * Plain pointers and sizes only. Every entry returns 0 on success or an error code
 * (MPSB_ERR_*) and leaves a thread-local message for mpsb_cuda_last_error(). The error
 * classes mirror the reference's exceptions: TrainingError (objective.hpp:17-20),
 * DataError (binned_dataset.hpp:18-21) and BackendError (backend.hpp:22-25).
 *
 * Reference interfaces each entry replaces (paths inside the reference project):
 *   mpsb_cuda_backend_create/destroy   MpsBackend::MpsBackend / ~MpsBackend
 *                                      (include/mpsboost/backend.hpp:140-150)
 *   mpsb_cuda_backend_info             QueryBackendInfo (backend.hpp:197-200)
 *   mpsb_quantize_dense                QuantizeDense (binned_dataset.hpp:137-138)
 *   mpsb_transform_dense               TransformDense (binned_dataset.hpp:140-144)
 *   mpsb_cuda_dataset_quantize         QuantizeDense (binned_dataset.hpp:137-138) on the
 *                                      device, the binned matrix left resident
 *   mpsb_cuda_dataset_transform        TransformDense (binned_dataset.hpp:140-144) on
 *                                      the device with a quantized dataset's schema
 *   mpsb_cuda_dataset_create           the per-node NewBuffer(dataset.bin_data())
 *                                      upload of src/mps/mps_histogram.mm:149, made
 *                                      once per dataset and kept resident
 *   mpsb_cuda_dataset_create_async     the same upload left in flight, so the caller's
 *   mpsb_cuda_dataset_wait             host work (label and weight checks) overlaps it
 *   mpsb_cuda_squared_error            GradientComputer::ComputeSquaredError
 *                                      (backend.hpp:52-58)
 *   mpsb_cuda_build_histograms         HistogramBuilder::BuildHistograms
 *                                      (backend.hpp:64-75)
 *   mpsb_cuda_build_layer_histograms   LayerHistogramBuilder::BuildLayerHistograms
 *                                      (backend.hpp:124-135)
 *   mpsb_cuda_scan_splits              MpsBackend::ScanSplitsForTest
 *                                      (backend.hpp:173-180), with the full
 *                                      FindBestSplit semantics (tree_split.cpp:142-234)
 *   mpsb_cuda_partition_rows           MpsBackend::PartitionRowsForTest
 *                                      (backend.hpp:181-185), with missing rows
 *                                      routed by default_left (tree_split.cpp:273-285)
 *   mpsb_cuda_train_regressor          TrainRegressionModel (trainer.hpp:133-139) as
 *                                      called by _train_regressor_mps
 *                                      (src/python/binding_model.cpp:34-45)
 *   mpsb_cuda_train_ovr                the one-vs-rest fit of
 *                                      src/mpsboost/estimators/multiclass.py:113-160
 *   mpsb_cuda_train_softmax            TrainMulticlassSoftmaxModel (trainer.hpp:141-147)
 *   mpsb_cuda_model_predict_margins    MulticlassModel::PredictMargins
 *                                      (multiclass_trainer.cpp:212-235)
 *   mpsb_cuda_train_forest             the per-tree fits of _ForestMixin.fit
 *                                      (src/mpsboost/estimators/forest.py:101-183,
 *                                      forest_sampling.py:42-63): one single-round tree
 *                                      per row sample and feature subset
 *   mpsb_cuda_model_create             RegressionModel::Restore (trainer.hpp:271-279)
 *   mpsb_cuda_model_serialize /        SerializeModel / DeserializeModel, SaveModelFile /
 *   _deserialize / _save / _load       LoadModelFile (trainer.hpp:152-160): the native
 *                                      model format 1.4 (src/io/model_format.cpp,
 *                                      model_payload.cpp), byte for byte
 *   mpsb_cuda_model_predict            RegressionModel::Predict (trainer.hpp:266-269)
 *   mpsb_cuda_trainer_*                the same training loop as a session with
 *                                      device-resident inputs (benchmarks, timing)
 */
#ifndef MPSB_CUDA_H
#define MPSB_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPSB_CUDA_ABI_VERSION 2

enum {
  MPSB_OK = 0,
  MPSB_ERR_TRAINING = 1, /* contract / math violation (TrainingError) */
  MPSB_ERR_DATA = 2,     /* input data violation (DataError) */
  MPSB_ERR_BACKEND = 3,  /* CUDA runtime / device failure (BackendError) */
  MPSB_ERR_UNSUPPORTED = 4
};

/* Objectives: TrainingParameters::Objective (trainer.hpp:21-27). */
enum { MPSB_SQUARED_ERROR = 0, MPSB_BINARY_LOGISTIC = 1, MPSB_QUANTILE = 2,
       MPSB_POISSON = 3, MPSB_TWEEDIE = 4 };

/* Histogram arithmetic. FIXED: FP32 g/h quantized per round to int64 with a power-of-two
   scale from max|g| and max h; exact, order-independent, deterministic sums. FLOAT: plain
   FP32 shared-memory atomics flushed into FP64 node histograms. */
enum { MPSB_HIST_FIXED = 0, MPSB_HIST_FLOAT = 1 };

/* Trainer option bits. */
enum {
  MPSB_OPT_FLOAT_HIST = 1u << 0, /* use MPSB_HIST_FLOAT */
  MPSB_OPT_NO_GRAPH = 1u << 1,   /* launch each round's kernels directly (no CUDA graph) */
  MPSB_OPT_PER_NODE = 1u << 2,   /* one histogram launch per node and a host round trip
                                    per level: the shape of mps_histogram.mm:62-80 */
  MPSB_OPT_TIMING = 1u << 3      /* CUDA events around every histogram launch */
};

/* TrainingParameters + TreeTrainingParameters (trainer.hpp:20-36, tree.hpp:47-72). */
typedef struct {
  uint32_t n_estimators;
  uint32_t max_bins;
  uint32_t objective;
  uint32_t max_depth;
  uint32_t max_leaves;
  uint32_t max_active_leaves;
  uint32_t split_strategy;  /* 0 best_gain, 1 random_threshold */
  uint32_t growth_strategy; /* 0 level_wise (1 leaf_wise is not provided here) */
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
  const int8_t* monotonic_constraints;  /* n_monotonic entries or NULL */
  const uint32_t* interaction_offsets;  /* n_interaction_groups + 1 entries */
  const uint32_t* interaction_features; /* concatenated groups */
} mpsb_train_params;

/* TreeNode (tree.hpp:31-42); 40 bytes. */
typedef struct {
  uint32_t feature_index;
  uint32_t threshold_bin;
  uint32_t left_child;
  uint32_t right_child;
  double leaf_value;
  double gain;
  uint8_t default_left;
  uint8_t flags; /* bit 0: leaf */
  uint8_t reserved[6];
} mpsb_tree_node;

/* HistogramBin (backend.hpp:40-44). */
typedef struct {
  uint64_t count;
  double gradient_sum;
  double hessian_sum;
} mpsb_histogram_bin;

/* SplitScanCandidate (backend.hpp:108-119) plus the chosen missing direction. */
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
} mpsb_split_candidate;

/* BackendInfo (backend.hpp:30-35) plus the device facts the kernels are sized by. */
typedef struct {
  uint32_t available;
  uint32_t sm_count;
  uint32_t cc_major;
  uint32_t cc_minor;
  uint64_t total_memory;
  char device_name[96];
} mpsb_cuda_info;

/* Per-kernel accounting of a trainer session (what one launch list shows). */
typedef struct {
  uint64_t rounds;
  uint64_t kernel_launches;    /* kernels of this library enqueued (graph nodes counted
                                  once per replay) */
  uint64_t hist_launches;      /* histogram-build launches */
  uint64_t hist_cells;         /* row x feature cells accumulated by histogram builds */
  uint64_t hist_rows;          /* rows gathered by histogram builds */
  double hist_ms;              /* summed CUDA-event time of histogram builds
                                  (MPSB_OPT_TIMING only) */
  uint64_t hist_timed_launches;
  uint64_t part_rows;          /* rows routed by row partitions (every split level but the
                                  last, whose rows go straight to the leaves) */
} mpsb_cuda_stats;

/* Launch shape of a training session: histogram CTA threads and pipeline stages,
   gradient-only root CTA threads, histogram work items per SM, depth levels built from
   the column-blocked bins copy, split-scan CTA threads. */
typedef struct {
  uint32_t hist_threads;
  uint32_t hist_stages;
  uint32_t root_threads;
  uint32_t items_per_sm;
  uint32_t blocked_levels;
  uint32_t scan_threads;
  double ms_per_round;          /* measured with this shape */
  double default_ms_per_round;  /* measured with the built-in shape */
  uint32_t trials;
} mpsb_cuda_tuning;

typedef struct mpsb_cuda_backend mpsb_cuda_backend;
typedef struct mpsb_cuda_dataset mpsb_cuda_dataset;
typedef struct mpsb_cuda_model mpsb_cuda_model;
typedef struct mpsb_cuda_trainer mpsb_cuda_trainer;

const char* mpsb_cuda_last_error(void);
int mpsb_cuda_abi_version(void);

/* ---- backend ------------------------------------------------------------------- */
/* Number of GPUs this library can train on (compute capability 10.3); 0 where there is no
   CUDA driver or device. Creates no context. The availability probe of the device policy
   (device_policy.py:64-99 asks diagnostics.is_available for MPS). */
int mpsb_cuda_device_count(int* out);
int mpsb_cuda_backend_create(int device, mpsb_cuda_backend** out);
void mpsb_cuda_backend_destroy(mpsb_cuda_backend* backend);
int mpsb_cuda_backend_info(const mpsb_cuda_backend* backend, mpsb_cuda_info* out);
/* Histogram arithmetic of the node-level entries below (MPSB_HIST_*); default FIXED. */
int mpsb_cuda_backend_set_hist_mode(mpsb_cuda_backend* backend, int mode);
/* CUDA-event timer on the backend's stream. */
int mpsb_cuda_timer_begin(mpsb_cuda_backend* backend);
int mpsb_cuda_timer_end(mpsb_cuda_backend* backend, float* milliseconds);
int mpsb_cuda_synchronize(mpsb_cuda_backend* backend);
/* Page-lock (pin) / release a caller-owned host buffer so copies from it run at full
   host-link bandwidth. */
int mpsb_cuda_host_register(void* ptr, uint64_t bytes);
int mpsb_cuda_host_unregister(void* ptr);

/* ---- binning (host) ------------------------------------------------------------- */
/* Quantile binning with the reference's semantics. scalar_type: 1 float32, 2 float64.
   Outputs are caller-allocated: bins [features*rows] feature-major (uint8 when
   max_bins <= 256, else uint16), missing [features*rows] (0/1), boundaries
   [features*(max_bins-1)] (used prefix = sum of boundary_count), boundary_offset,
   boundary_count, bin_count, missing_count [features]. n_threads 0 = all host cores. */
int mpsb_quantize_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                        uint64_t row_stride_bytes, uint64_t column_stride_bytes,
                        uint32_t max_bins, uint32_t n_threads, void* bins, uint8_t* missing,
                        float* boundaries, uint64_t* boundary_offset,
                        uint32_t* boundary_count, uint32_t* bin_count,
                        uint64_t* missing_count);
/* Apply an existing schema (boundaries/offsets/counts of mpsb_quantize_dense). */
int mpsb_transform_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                         uint64_t row_stride_bytes, uint64_t column_stride_bytes,
                         uint32_t max_bins, const float* boundaries,
                         const uint64_t* boundary_offset, const uint32_t* boundary_count,
                         uint32_t n_threads, void* bins, uint8_t* missing);

/* ---- device-resident dataset ------------------------------------------------------ */
/* bins: feature-major [features*rows], bin_width_bytes 1 or 2; missing may be NULL.
   Each feature needs 1 <= bin_count <= 65536, and <= 65535 when it has missing rows.
   When every feature's bins and missing slot fit in 256 histogram slots the dataset keeps
   u8 copies; otherwise (more than 256 bins, or 256 bins and missing rows) u16 copies and
   the wide kernels (about twice the time per tree at 512 slots). */
int mpsb_cuda_dataset_create(mpsb_cuda_backend* backend, const void* bins,
                             uint32_t bin_width_bytes, const uint8_t* missing,
                             uint64_t rows, uint32_t features, const uint32_t* bin_count,
                             mpsb_cuda_dataset** out);
/* As mpsb_cuda_dataset_create, but returns once the upload is enqueued. bins and missing
   must stay valid and unchanged until mpsb_cuda_dataset_wait, or the first entry that
   reads the dataset (training, prediction, histograms, export), has returned; a bin past
   its feature's count is reported there (MPSB_ERR_DATA) rather than here. */
int mpsb_cuda_dataset_create_async(mpsb_cuda_backend* backend, const void* bins,
                                   uint32_t bin_width_bytes, const uint8_t* missing,
                                   uint64_t rows, uint32_t features, const uint32_t* bin_count,
                                   mpsb_cuda_dataset** out);
/* Waits for an asynchronous upload to complete (returns at once for a complete one). */
int mpsb_cuda_dataset_wait(const mpsb_cuda_dataset* dataset);
void mpsb_cuda_dataset_destroy(mpsb_cuda_dataset* dataset);
/* 1 when the dataset's row-major bins carry a TMA tensor map (row-major histogram levels
   stage their gathered rows with tile::gather4 copies), else 0 (cp.async staging); set at
   creation when the environment variable MPSB_HIST_TMA is 1. */
int mpsb_cuda_dataset_uses_tma(const mpsb_cuda_dataset* dataset);

/* ---- node-level entries (the backend.hpp contract) ----------------------------------- */
int mpsb_cuda_squared_error(mpsb_cuda_backend* backend, const double* labels,
                            const double* predictions, uint64_t n, double* out_pairs);
/* pairs: [n_pairs][2] FP64 (GradientPair); out: features x bin_count bins; missing rows
   are counted in bin 0 as in the reference. */
int mpsb_cuda_build_histograms(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                               const uint64_t* rows, uint64_t n_rows, const double* pairs,
                               uint64_t n_pairs, mpsb_histogram_bin* out);
/* node_offsets: n_nodes+1 offsets into rows; out: n_nodes blocks of features x bin_count. */
int mpsb_cuda_build_layer_histograms(mpsb_cuda_backend* backend,
                                     const mpsb_cuda_dataset* dataset, const uint64_t* rows,
                                     const uint64_t* node_offsets, uint32_t n_nodes,
                                     const double* pairs, uint64_t n_pairs,
                                     mpsb_histogram_bin* out);
int mpsb_cuda_scan_splits(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                          const uint64_t* rows, uint64_t n_rows, const double* pairs,
                          uint64_t n_pairs, const mpsb_train_params* params,
                          mpsb_split_candidate* out_per_feature);
int mpsb_cuda_partition_rows(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                             const uint64_t* rows, uint64_t n_rows, uint32_t feature,
                             uint32_t threshold_bin, int default_left, uint64_t* left_out,
                             uint64_t* right_out, uint64_t* n_left);

/* Histogram build that allocates no device memory (no counterpart in the reference).
   For callers that must not call cudaMalloc -- a plugin inside a process whose device
   memory belongs to that process's own pool allocator, or a serving loop that cannot
   afford cudaMalloc's implicit synchronisation. All inputs and the output are the
   caller's device buffers:
     bins   column-blocked u8 [ceil(features/32)][dataset_rows][32] (feature f of row r at
            ((f/32)*dataset_rows + r)*32 + f%32; padding features 0; a missing value may
            use bin 255 and then lands in slot 255),
     rows   u32 [n_rows] row ids of the node (< dataset_rows),
     pairs  FP32 [dataset_rows][2] gradient/hessian pairs, all finite, hessians >= 0 (the
            scale comes from every row's pair, not only the node's); if any pair breaks
            this, no histogram is built and every bin of `out` gets count 0 and NaN sums,
            since the entry cannot report an error without waiting for the GPU,
     out    [features][256] bins: exact fixed-point count/G/H as FP64 (same scale rule and
            kernel as mpsb_cuda_build_histograms).
   Work is enqueued on `stream` (a cudaStream_t; NULL = default stream) and not waited for.
   Intermediates live in a fixed 2 MiB array inside the library that every GPU keeps
   until the process exits; features above 256 are rejected. The first call on a device
   looks the array up (make it before any stream capture); every call shares the array,
   so calls that overlap on the GPU race. */
int mpsb_cuda_build_histogram_noalloc(const uint8_t* bins, uint32_t dataset_rows,
                                      uint32_t features, const uint32_t* rows,
                                      uint32_t n_rows, const float* pairs,
                                      mpsb_histogram_bin* out, void* stream);

/* ---- quantile binning on the device ------------------------------------------- */
/* QuantizeDense on the GPU: the matrix (scalar_type 1 = float32, 2 = float64; element
   (r, f) at byte offset r * row_stride + f * col_stride) is uploaded, binned with the
   reference's quantile rule and kept resident as a training dataset. NaN is missing, Inf
   and float64 values outside the float32 range are DataErrors. max_bins in [2, 65536]
   (a feature with 65536 bins may not have missing values); above 256 the order
   statistics come from a per-feature sort. Bins and boundaries equal
   mpsb_quantize_dense's, except that a boundary at zero may carry either sign (the two
   zeros compare equal). */
int mpsb_cuda_dataset_quantize(mpsb_cuda_backend* backend, const void* data, int scalar_type,
                               uint64_t rows, uint32_t features, uint64_t row_stride,
                               uint64_t col_stride, uint32_t max_bins, mpsb_cuda_dataset** out);
/* TransformDense on the GPU with the boundaries of a device-quantized dataset. */
int mpsb_cuda_dataset_transform(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* schema,
                                const void* data, int scalar_type, uint64_t rows,
                                uint32_t features, uint64_t row_stride, uint64_t col_stride,
                                mpsb_cuda_dataset** out);
/* The schema of a device-quantized dataset: boundary_total() floats, and per feature the
   offset and count of its boundaries, its bin count and missing count. Any output may be
   NULL. */
uint64_t mpsb_cuda_dataset_boundary_total(const mpsb_cuda_dataset* dataset);
int mpsb_cuda_dataset_schema(const mpsb_cuda_dataset* dataset, float* boundaries,
                             uint64_t* boundary_offset, uint32_t* boundary_count,
                             uint32_t* bin_count, uint64_t* missing_count);
/* The binned matrix, feature-major u8 [features][rows] (missing rows as bin 0), and the
   missing flags (may be NULL), as mpsb_quantize_dense lays them out; UnsupportedError for
   a dataset with more than 256 bins in a feature. */
int mpsb_cuda_dataset_export(const mpsb_cuda_dataset* dataset, uint8_t* bins, uint8_t* missing);
/* The same as u16 [features][rows], for any dataset (mpsb_quantize_dense's layout when
   max_bins > 256). */
int mpsb_cuda_dataset_export16(const mpsb_cuda_dataset* dataset, uint16_t* bins, uint8_t* missing);

/* Softmax models: class count (0 for a regression model), base scores, margins
   [rows][class_count] of a binned dataset, and creation from host trees ordered
   (round, class). */
uint32_t mpsb_cuda_model_class_count(const mpsb_cuda_model* model);
int mpsb_cuda_model_class_base_scores(const mpsb_cuda_model* model, double* out);
int mpsb_cuda_model_predict_margins(mpsb_cuda_backend* backend, const mpsb_cuda_model* model,
                                    const mpsb_cuda_dataset* dataset, double* out);
int mpsb_cuda_model_class_labels(const mpsb_cuda_model* model, double* out);
/* class_labels may be NULL (0..class_count-1); otherwise strictly increasing. */
int mpsb_cuda_model_create_softmax(uint32_t class_count, double learning_rate,
                                   const double* base_scores, const double* class_labels,
                                   uint32_t n_trees, const uint32_t* node_counts,
                                   const mpsb_tree_node* nodes, mpsb_cuda_model** out);

/* ---- model files ----------------------------------------------------------------- */
/* The reference's native model format (magic MPSBMOD, version 1.4, FNV-1a checksum),
   byte for byte: models written here load in the reference and the reference's load
   here (minor versions 0-4 are read). A model needs its training data's quantization
   schema (softmax models are written as the multiclass kind):
   models trained on a device-quantized dataset carry it; otherwise attach it
   with mpsb_cuda_model_set_schema (the arrays of mpsb_quantize_dense). Objective
   metadata comes from training (or mpsb_cuda_model_set_objective). Reading applies the
   reference's validation; violations are TrainingErrors (DataError for the schema). */
int mpsb_cuda_model_set_schema(mpsb_cuda_model* model, uint32_t features, uint32_t max_bins,
                               const float* boundaries, uint64_t n_boundaries,
                               const uint64_t* boundary_offset, const uint32_t* boundary_count,
                               const uint32_t* bin_count, const uint64_t* missing_count);
int mpsb_cuda_model_set_objective(mpsb_cuda_model* model, uint32_t objective, double alpha,
                                  double variance_power);
int mpsb_cuda_model_get_objective(const mpsb_cuda_model* model, uint32_t* objective,
                                  double* alpha, double* variance_power);
/* Sizes first (array outputs NULL), then the arrays. */
int mpsb_cuda_model_get_schema(const mpsb_cuda_model* model, uint32_t* features,
                               uint32_t* max_bins, uint64_t* n_boundaries, float* boundaries,
                               uint64_t* boundary_offset, uint32_t* boundary_count,
                               uint32_t* bin_count, uint64_t* missing_count);
/* *size receives the file size; out (capacity bytes) receives the bytes when not NULL. */
int mpsb_cuda_model_serialize(const mpsb_cuda_model* model, uint8_t* out, uint64_t capacity,
                              uint64_t* size);
/* kind: 0 = DeserializeModel (regression files only), 1 = DeserializeMulticlassModel
   (multiclass files only), -1 = either. */
int mpsb_cuda_model_deserialize(const uint8_t* data, uint64_t size, int kind,
                                mpsb_cuda_model** out);
/* Atomic save (temporary file in the same directory, fsync, rename) and load. */
int mpsb_cuda_model_save(const mpsb_cuda_model* model, const char* path);
int mpsb_cuda_model_load(const char* path, int kind, mpsb_cuda_model** out);

/* ---- training ------------------------------------------------------------------ */
/* weights may be NULL (unit weights). options: MPSB_OPT_* bits. */
int mpsb_cuda_train_regressor(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                              const double* labels, const double* weights, uint64_t n,
                              const mpsb_train_params* params, uint32_t options,
                              mpsb_cuda_model** out);
/* K binary-logistic models on labels (class ids 0..K-1), all K trees of a round built in
   the same launches. out receives K models. */
int mpsb_cuda_train_ovr(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                        const double* labels, const double* weights, uint64_t n,
                        uint32_t n_classes, const mpsb_train_params* params,
                        uint32_t options, mpsb_cuda_model** out);
/* Native softmax boosting: per round one tree per class, in class order, each fitted to
   the softmax gradients of the current margins (which include the earlier classes' trees
   of the round). labels are class ids 0..class_count-1. The model holds class_count base
   scores (log class priors), the trees ordered (round, class) and, as its training
   predictions, the margins [n][class_count]. */
int mpsb_cuda_train_softmax(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                            const double* labels, const double* weights, uint64_t n,
                            const mpsb_train_params* params, uint32_t class_count,
                            uint32_t options, mpsb_cuda_model** out);
/* n_trees independent single-round trees (a random forest / extra-trees ensemble), the
   frontier of every tree of a batch built in the same launches. Tree t trains on the
   multiset of rows given by row_counts[t * n + r] (how many times row r is drawn: 0 for
   rows outside the bootstrap sample) and on the features
   features[feature_offsets[t] .. feature_offsets[t + 1]); the result equals the
   reference's fit on matrix[rows][:, sorted(features)] with this dataset's bins (ties
   between features resolve by feature index). seeds[t] (or params->random_seed when
   seeds is NULL) seeds random thresholds; a feature's rank in the tree's ascending
   subset enters the threshold hash. params->n_estimators is ignored; interaction
   constraints are unsupported. out receives n_trees models of one tree each, without
   training predictions. */
int mpsb_cuda_train_forest(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                           const double* labels, const double* weights, uint64_t n,
                           const mpsb_train_params* params, uint32_t n_trees,
                           const uint8_t* row_counts, const uint32_t* feature_offsets,
                           const uint32_t* features, const uint32_t* seeds, uint32_t options,
                           mpsb_cuda_model** out);
/* A model from host trees (e.g. one loaded from a file): base_score + learning_rate *
   sum of trees, node_counts[n_trees], nodes concatenated tree by tree. */
int mpsb_cuda_model_create(double base_score, double learning_rate, uint32_t n_trees,
                           const uint32_t* node_counts, const mpsb_tree_node* nodes,
                           mpsb_cuda_model** out);
uint32_t mpsb_cuda_model_tree_count(const mpsb_cuda_model* model);
double mpsb_cuda_model_base_score(const mpsb_cuda_model* model);
double mpsb_cuda_model_learning_rate(const mpsb_cuda_model* model);
uint32_t mpsb_cuda_model_tree_node_count(const mpsb_cuda_model* model, uint32_t tree);
int mpsb_cuda_model_tree_nodes(const mpsb_cuda_model* model, uint32_t tree,
                               mpsb_tree_node* out);
/* Final FP64 training predictions (base + lr * sum of leaves) kept by the trainer. */
int mpsb_cuda_model_train_predictions(const mpsb_cuda_model* model, double* out);
int mpsb_cuda_model_predict(mpsb_cuda_backend* backend, const mpsb_cuda_model* model,
                            const mpsb_cuda_dataset* dataset, double* out);
void mpsb_cuda_model_destroy(mpsb_cuda_model* model);

/* ---- training session (device-resident inputs; benchmarks) ---------------------------- */
int mpsb_cuda_trainer_create(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                             const double* labels, const double* weights, uint64_t n,
                             const mpsb_train_params* params, uint32_t options,
                             mpsb_cuda_trainer** out);
/* Enqueue `rounds` boosting rounds on the backend stream (asynchronous). */
int mpsb_cuda_trainer_run(mpsb_cuda_trainer* trainer, uint32_t rounds);
/* Wait for the stream and report any device-side error. */
int mpsb_cuda_trainer_synchronize(mpsb_cuda_trainer* trainer);
int mpsb_cuda_trainer_stats(const mpsb_cuda_trainer* trainer, mpsb_cuda_stats* out);
int mpsb_cuda_trainer_reset_stats(mpsb_cuda_trainer* trainer);
/* Per depth level (MPSB_OPT_TIMING): summed histogram-build milliseconds and cells since
   the last reset; n_levels entries are written (levels beyond the tree depth get 0). */
int mpsb_cuda_trainer_level_stats(const mpsb_cuda_trainer* trainer, uint32_t n_levels,
                                  double* milliseconds, uint64_t* cells);
int mpsb_cuda_trainer_export(mpsb_cuda_trainer* trainer, mpsb_cuda_model** out);

/* Autotuner: times boosting rounds of this fit's shape (rows, features, depth, histogram
   arithmetic, weighted or not, growth strategy) under launch shapes chosen by coordinate
   descent from the built-in one (rounds_per_trial timed rounds each, after one untimed),
   and keeps the fastest in a process-wide table that every later session of the same
   shape uses (the MPSB_* tile variables still override it). Results do not depend on
   the shape: every launch shape gives the same trees. */
int mpsb_cuda_autotune(mpsb_cuda_backend* backend, const mpsb_cuda_dataset* dataset,
                       const double* labels, const double* weights, uint64_t n,
                       const mpsb_train_params* params, uint32_t options,
                       uint32_t rounds_per_trial, mpsb_cuda_tuning* out);
/* Forget every tuned shape. */
void mpsb_cuda_autotune_clear(void);
void mpsb_cuda_trainer_destroy(mpsb_cuda_trainer* trainer);

#ifdef __cplusplus
}
#endif

#endif
