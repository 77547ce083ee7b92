/*
 * Plain-C restatement of the MPSBoost GBDT training hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the CPU oracle the CUDA backend is checked against. It is never linked
 * into the product; only tests, the smoke check and the benchmark's CPU-baseline leg
 * load it. Every function names the reference file:line it restates. Two histogram
 * modes grow trees:
 *   ORC_HIST_FP64  - the reference exactly: FP64 gradients, FP64 sums in row order,
 *                    FP64 subtraction with the Hessian clamp, sequential FP64 prefix scan.
 *   ORC_HIST_FIXED - the replica of the CUDA fixed-point path: each round's weighted
 *                    FP64 gradients are rounded to FP32, quantized to int64 with a
 *                    power-of-two scale taken from max|g| and max h, summed exactly;
 *                    prefix sums and statistics stay int64 and are converted to FP64
 *                    only where the reference evaluates gains and leaf values.
 * The pinning of this file against the compiled reference is in tests/test_oracle_pin.py.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static __thread char g_err[512];

/* Threads of the feature-parallel loops (histograms, missing statistics). Every bin is
 * owned by one feature and summed in row order whatever the thread count, so results do
 * not depend on it; 1 reproduces the reference's single-threaded timing. */
static int g_threads = 0; /* 0: OpenMP's default (all cores) */
void orc_set_threads(int threads) { g_threads = threads > 0 ? threads : 0; }
static int n_threads(uint64_t work) {
  if (work < (1u << 20)) return 1; /* small nodes: not worth a parallel region */
  return g_threads > 0 ? g_threads : omp_get_max_threads();
}

static int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

#define TRY(expr)                \
  do {                           \
    int rc_ = (expr);            \
    if (rc_ != ORC_OK) return rc_; \
  } while (0)

const char* orc_last_error(void) { return g_err; }

/* ------------------------------------------------------------------------------------
 * Binned dataset: feature-major bins + missing mask + schema
 * (binned_dataset.hpp:81-126, binned_dataset.cpp:126-238)
 * ---------------------------------------------------------------------------------- */
typedef struct {
  uint64_t rows;
  uint32_t features;
  uint32_t max_bins;
  float* boundaries;
  uint64_t n_boundaries;
  uint64_t* boundary_offset;
  uint32_t* boundary_count;
  uint32_t* bin_count;
  uint64_t* missing_count;
  uint16_t* bins;    /* [features][rows] */
  uint8_t* missing;  /* [features][rows] */
} dataset_t;

void orc_dataset_free(void* p) {
  dataset_t* d = (dataset_t*)p;
  if (d == NULL) return;
  free(d->boundaries);
  free(d->boundary_offset);
  free(d->boundary_count);
  free(d->bin_count);
  free(d->missing_count);
  free(d->bins);
  free(d->missing);
  free(d);
}

/* ValidateViewImpl, binned_dataset.cpp:19-48 (overflow checks restated with builtins). */
static int validate_view(const void* data, int scalar_type, uint64_t rows,
                         uint32_t features, uint64_t rs, uint64_t cs, uint32_t max_bins) {
  if (data == NULL) return fail(ORC_DATA_ERROR, "Input matrix data must not be null");
  if (rows == 0 || features == 0)
    return fail(ORC_DATA_ERROR, "Input matrix must contain at least one row and one feature");
  if (max_bins < 2 || max_bins > 65536)
    return fail(ORC_DATA_ERROR, "max_bins must be in [2, 65536]");
  if (scalar_type != 1 && scalar_type != 2)
    return fail(ORC_DATA_ERROR, "Input scalar type is not supported");
  const uint64_t item = scalar_type == 2 ? 8 : 4;
  if (rs < item || cs < item)
    return fail(ORC_DATA_ERROR, "Input matrix stride is smaller than the element size");
  uint64_t a, b, c;
  if (__builtin_mul_overflow(rows - 1, rs, &a) ||
      __builtin_mul_overflow((uint64_t)(features - 1), cs, &b) ||
      __builtin_add_overflow(a, b, &c) || __builtin_add_overflow(c, item, &c) ||
      __builtin_mul_overflow(rows, (uint64_t)features, &a))
    return fail(ORC_DATA_ERROR, "input matrix maximum offset: multiplication overflow");
  return ORC_OK;
}

/* ReadFiniteOrMissingFloat, binned_dataset.cpp:50-81. */
static int read_value(const void* data, int scalar_type, uint64_t rs, uint64_t cs,
                      uint64_t row, uint32_t feature, float* out) {
  const uint8_t* address = (const uint8_t*)data + row * rs + (uint64_t)feature * cs;
  if (scalar_type == 1) {
    float v;
    memcpy(&v, address, sizeof v);
    if (isnan(v)) { *out = v; return ORC_OK; }
    if (!isfinite(v)) return fail(ORC_DATA_ERROR, "Input matrix contains Inf");
    *out = v;
    return ORC_OK;
  }
  double s;
  memcpy(&s, address, sizeof s);
  if (isnan(s)) { *out = NAN; return ORC_OK; }
  if (!isfinite(s)) return fail(ORC_DATA_ERROR, "Input matrix contains Inf");
  if (s > (double)FLT_MAX || s < -(double)FLT_MAX)
    return fail(ORC_DATA_ERROR, "float64 input value exceeds the finite float32 range");
  *out = (float)s;
  return ORC_OK;
}

/* QuantileRank, binned_dataset.cpp:83-93: ceil(part * total / divisor) - 1 without overflow. */
static uint64_t quantile_rank(uint64_t part, uint64_t total, uint64_t divisor) {
  const uint64_t quotient = total / divisor;
  const uint64_t remainder = total % divisor;
  const uint64_t whole = part * quotient;
  const uint64_t numerator = part * remainder;
  const uint64_t fraction = numerator / divisor + (numerator % divisor != 0 ? 1 : 0);
  return whole + fraction - 1;
}

static int cmp_float(const void* a, const void* b) {
  const float x = *(const float*)a, y = *(const float*)b;
  return (x > y) - (x < y);
}

/* BuildBoundaries, binned_dataset.cpp:95-118. `values` is scratch (NaN allowed). */
static uint32_t build_boundaries(float* values, uint64_t n, uint32_t max_bins, float* out) {
  uint64_t m = 0;
  for (uint64_t i = 0; i < n; ++i)
    if (!isnan(values[i])) values[m++] = values[i];
  if (m == 0) return 0;
  qsort(values, m, sizeof(float), cmp_float);
  const uint64_t desired = m < max_bins ? m : max_bins;
  const float maximum = values[m - 1];
  uint32_t count = 0;
  for (uint64_t part = 1; part < desired; ++part) {
    const float candidate = values[quantile_rank(part, m, desired)];
    if (candidate < maximum && (count == 0 || candidate > out[count - 1]))
      out[count++] = candidate;
  }
  return count;
}

/* std::lower_bound over a feature's boundaries: first index with b[i] >= value. */
static uint32_t lower_bound_f(const float* b, uint32_t n, float value) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (b[mid] < value) lo = mid + 1; else hi = mid;
  }
  return lo;
}

static dataset_t* alloc_dataset(uint64_t rows, uint32_t features) {
  dataset_t* d = (dataset_t*)calloc(1, sizeof(dataset_t));
  if (d == NULL) return NULL;
  d->rows = rows;
  d->features = features;
  d->boundary_offset = (uint64_t*)calloc(features, sizeof(uint64_t));
  d->boundary_count = (uint32_t*)calloc(features, sizeof(uint32_t));
  d->bin_count = (uint32_t*)calloc(features, sizeof(uint32_t));
  d->missing_count = (uint64_t*)calloc(features, sizeof(uint64_t));
  d->bins = (uint16_t*)calloc(rows * features, sizeof(uint16_t));
  d->missing = (uint8_t*)calloc(rows * features, 1);
  if (!d->boundary_offset || !d->boundary_count || !d->bin_count || !d->missing_count ||
      !d->bins || !d->missing) {
    orc_dataset_free(d);
    return NULL;
  }
  return d;
}

/* QuantizeDense, binned_dataset.cpp:126-188. */
int orc_quantize_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                       uint64_t rs, uint64_t cs, uint32_t max_bins, void** out) {
  TRY(validate_view(data, scalar_type, rows, features, rs, cs, max_bins));
  dataset_t* d = alloc_dataset(rows, features);
  float* values = (float*)malloc(rows * sizeof(float));
  float* scratch = (float*)malloc(rows * sizeof(float));
  float* all = (float*)malloc(((uint64_t)features * (max_bins - 1) + 1) * sizeof(float));
  if (!d || !values || !scratch || !all) {
    orc_dataset_free(d); free(values); free(scratch); free(all);
    return fail(ORC_OTHER_ERROR, "out of host memory");
  }
  d->max_bins = max_bins;
  uint64_t total = 0;
  int rc = ORC_OK;
  for (uint32_t f = 0; f < features && rc == ORC_OK; ++f) {
    uint64_t missing = 0;
    for (uint64_t r = 0; r < rows; ++r) {
      rc = read_value(data, scalar_type, rs, cs, r, f, &values[r]);
      if (rc != ORC_OK) break;
      if (isnan(values[r])) ++missing;
    }
    if (rc != ORC_OK) break;
    memcpy(scratch, values, rows * sizeof(float));
    float* b = all + total;
    const uint32_t nb = build_boundaries(scratch, rows, max_bins, b);
    d->boundary_offset[f] = total;
    d->boundary_count[f] = nb;
    d->bin_count[f] = nb + 1;
    d->missing_count[f] = missing;
    for (uint64_t r = 0; r < rows; ++r) {
      const int is_missing = isnan(values[r]);
      d->missing[(uint64_t)f * rows + r] = (uint8_t)is_missing;
      d->bins[(uint64_t)f * rows + r] = (uint16_t)(is_missing ? 0 : lower_bound_f(b, nb, values[r]));
    }
    total += nb;
  }
  free(values);
  free(scratch);
  if (rc != ORC_OK) { orc_dataset_free(d); free(all); return rc; }
  d->n_boundaries = total;
  d->boundaries = (float*)realloc(all, (total > 0 ? total : 1) * sizeof(float));
  *out = d;
  return ORC_OK;
}

/* TransformDense, binned_dataset.cpp:190-238 (schema taken from a quantized dataset). */
int orc_transform_dense(const void* schema_dataset, const void* data, int scalar_type,
                        uint64_t rows, uint32_t features, uint64_t rs, uint64_t cs,
                        void** out) {
  const dataset_t* s = (const dataset_t*)schema_dataset;
  TRY(validate_view(data, scalar_type, rows, features, rs, cs, s->max_bins));
  if (features != s->features)
    return fail(ORC_DATA_ERROR, "Prediction input feature count does not match the binned schema");
  dataset_t* d = alloc_dataset(rows, features);
  if (!d) return fail(ORC_OTHER_ERROR, "out of host memory");
  d->max_bins = s->max_bins;
  d->n_boundaries = s->n_boundaries;
  d->boundaries = (float*)malloc((s->n_boundaries > 0 ? s->n_boundaries : 1) * sizeof(float));
  memcpy(d->boundaries, s->boundaries, s->n_boundaries * sizeof(float));
  memcpy(d->boundary_offset, s->boundary_offset, features * sizeof(uint64_t));
  memcpy(d->boundary_count, s->boundary_count, features * sizeof(uint32_t));
  memcpy(d->bin_count, s->bin_count, features * sizeof(uint32_t));
  memcpy(d->missing_count, s->missing_count, features * sizeof(uint64_t));
  for (uint32_t f = 0; f < features; ++f) {
    const float* b = s->boundaries + s->boundary_offset[f];
    for (uint64_t r = 0; r < rows; ++r) {
      float v;
      int rc = read_value(data, scalar_type, rs, cs, r, f, &v);
      if (rc != ORC_OK) { orc_dataset_free(d); return rc; }
      const int is_missing = isnan(v);
      d->missing[(uint64_t)f * rows + r] = (uint8_t)is_missing;
      d->bins[(uint64_t)f * rows + r] =
          (uint16_t)(is_missing ? 0 : lower_bound_f(b, s->boundary_count[f], v));
    }
  }
  *out = d;
  return ORC_OK;
}

int orc_dataset_subset(const void* src, const uint64_t* rows, uint64_t n_rows,
                       const uint32_t* features, uint32_t n_features, void** out) {
  const dataset_t* s = (const dataset_t*)src;
  if (n_rows == 0 || n_features == 0) return fail(ORC_DATA_ERROR, "empty subset");
  for (uint64_t i = 0; i < n_rows; ++i)
    if (rows[i] >= s->rows) return fail(ORC_DATA_ERROR, "subset row out of range");
  uint64_t total = 0;
  for (uint32_t j = 0; j < n_features; ++j) {
    if (features[j] >= s->features) return fail(ORC_DATA_ERROR, "subset feature out of range");
    total += s->boundary_count[features[j]];
  }
  dataset_t* d = alloc_dataset(n_rows, n_features);
  if (!d) return fail(ORC_OTHER_ERROR, "out of host memory");
  d->max_bins = s->max_bins;
  d->n_boundaries = total;
  d->boundaries = (float*)malloc((total > 0 ? total : 1) * sizeof(float));
  if (!d->boundaries) { orc_dataset_free(d); return fail(ORC_OTHER_ERROR, "out of host memory"); }
  uint64_t off = 0;
  for (uint32_t j = 0; j < n_features; ++j) {
    const uint32_t f = features[j];
    d->boundary_offset[j] = off;
    d->boundary_count[j] = s->boundary_count[f];
    d->bin_count[j] = s->bin_count[f];
    memcpy(d->boundaries + off, s->boundaries + s->boundary_offset[f],
           s->boundary_count[f] * sizeof(float));
    off += s->boundary_count[f];
    uint64_t missing = 0;
    for (uint64_t i = 0; i < n_rows; ++i) {
      const uint64_t si = (uint64_t)f * s->rows + rows[i], di = (uint64_t)j * n_rows + i;
      d->bins[di] = s->bins[si];
      d->missing[di] = s->missing[si];
      missing += s->missing[si];
    }
    d->missing_count[j] = missing;
  }
  *out = d;
  return ORC_OK;
}

/* A dataset from bins computed elsewhere under a known schema: the fields QuantizeDense
 * produces (binned_dataset.hpp:81-126), feature-major. Every non-missing bin must lie
 * below its feature's bin count; missing counts are recomputed. */
int orc_dataset_from_bins(const void* bins, uint32_t width, const uint8_t* missing,
                          uint64_t rows, uint32_t features, uint32_t max_bins,
                          const float* boundaries, const uint64_t* boundary_offset,
                          const uint32_t* boundary_count, const uint32_t* bin_count, void** out) {
  if (bins == NULL || boundary_offset == NULL || boundary_count == NULL || bin_count == NULL || out == NULL)
    return fail(ORC_DATA_ERROR, "null argument");
  if (width != 1 && width != 2) return fail(ORC_DATA_ERROR, "bin width must be 1 or 2 bytes");
  if (rows == 0 || features == 0) return fail(ORC_DATA_ERROR, "empty dataset");
  if (max_bins < 2 || max_bins > 65536) return fail(ORC_DATA_ERROR, "max_bins must be in [2, 65536]");
  uint64_t total = 0;
  for (uint32_t f = 0; f < features; ++f) {
    if (bin_count[f] == 0 || bin_count[f] > max_bins || boundary_count[f] + 1 != bin_count[f])
      return fail(ORC_DATA_ERROR, "bin counts do not match the boundaries");
    if (boundary_offset[f] != total) return fail(ORC_DATA_ERROR, "boundary offsets are not packed");
    total += boundary_count[f];
  }
  if (total > 0 && boundaries == NULL) return fail(ORC_DATA_ERROR, "null boundaries");
  dataset_t* d = alloc_dataset(rows, features);
  if (!d) return fail(ORC_OTHER_ERROR, "out of host memory");
  d->max_bins = max_bins;
  d->n_boundaries = total;
  d->boundaries = (float*)malloc((total > 0 ? total : 1) * sizeof(float));
  if (!d->boundaries) { orc_dataset_free(d); return fail(ORC_OTHER_ERROR, "out of host memory"); }
  if (total > 0) memcpy(d->boundaries, boundaries, total * sizeof(float));
  for (uint32_t f = 0; f < features; ++f) {
    d->boundary_offset[f] = boundary_offset[f];
    d->boundary_count[f] = boundary_count[f];
    d->bin_count[f] = bin_count[f];
    uint64_t miss = 0;
    for (uint64_t r = 0; r < rows; ++r) {
      const uint64_t i = (uint64_t)f * rows + r;
      const uint32_t b = width == 1 ? ((const uint8_t*)bins)[i] : ((const uint16_t*)bins)[i];
      const uint8_t m = missing ? (missing[i] != 0) : 0;
      if (!m && b >= bin_count[f]) {
        orc_dataset_free(d);
        return fail(ORC_DATA_ERROR, "Binned value exceeds the feature histogram range");
      }
      d->bins[i] = (uint16_t)(m ? 0 : b);
      d->missing[i] = m;
      miss += m;
    }
    d->missing_count[f] = miss;
  }
  *out = d;
  return ORC_OK;
}

int orc_dataset_info(const void* p, uint64_t* rows, uint32_t* features, uint32_t* max_bins,
                     uint64_t* boundary_total) {
  const dataset_t* d = (const dataset_t*)p;
  *rows = d->rows;
  *features = d->features;
  *max_bins = d->max_bins;
  *boundary_total = d->n_boundaries;
  return ORC_OK;
}

int orc_dataset_metadata(const void* p, uint64_t* off, uint32_t* cnt, uint32_t* bins,
                         uint64_t* miss) {
  const dataset_t* d = (const dataset_t*)p;
  memcpy(off, d->boundary_offset, d->features * sizeof(uint64_t));
  memcpy(cnt, d->boundary_count, d->features * sizeof(uint32_t));
  memcpy(bins, d->bin_count, d->features * sizeof(uint32_t));
  memcpy(miss, d->missing_count, d->features * sizeof(uint64_t));
  return ORC_OK;
}

int orc_dataset_boundaries(const void* p, float* out) {
  const dataset_t* d = (const dataset_t*)p;
  memcpy(out, d->boundaries, d->n_boundaries * sizeof(float));
  return ORC_OK;
}

int orc_dataset_bins(const void* p, uint16_t* out) {
  const dataset_t* d = (const dataset_t*)p;
  memcpy(out, d->bins, d->rows * d->features * sizeof(uint16_t));
  return ORC_OK;
}

int orc_dataset_missing(const void* p, uint8_t* out) {
  const dataset_t* d = (const dataset_t*)p;
  memcpy(out, d->missing, d->rows * d->features);
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------
 * Objectives (objective.cpp:101-287) and the trainer's weighting (trainer.cpp:178-216)
 * ---------------------------------------------------------------------------------- */
static int safe_exp(double v, const char* field, double* out) { /* objective.cpp:252-262 */
  if (!isfinite(v)) return fail(ORC_TRAINING_ERROR, "%s must be finite", field);
  if (v > 709.0) return fail(ORC_TRAINING_ERROR, "%s exponential overflowed", field);
  *out = exp(v);
  if (!isfinite(*out)) return fail(ORC_TRAINING_ERROR, "%s exponential overflowed", field);
  return ORC_OK;
}

static double logistic_probability(double logit) { /* objective.cpp:309-317 */
  if (logit >= 0.0) {
    const double e = exp(-logit);
    return 1.0 / (1.0 + e);
  }
  const double e = exp(logit);
  return e / (1.0 + e);
}

int orc_gradients(uint32_t objective, double alpha, double tvp, const double* labels,
                  const double* preds, uint64_t n, double* out) {
  if (n == 0) return fail(ORC_TRAINING_ERROR, "Labels must not be empty");
  if (objective == ORC_QUANTILE && (!isfinite(alpha) || alpha <= 0.0 || alpha >= 1.0))
    return fail(ORC_TRAINING_ERROR, "quantile alpha must be in (0, 1)");
  if (objective == ORC_TWEEDIE && (!isfinite(tvp) || tvp <= 1.0 || tvp >= 2.0))
    return fail(ORC_TRAINING_ERROR, "tweedie variance power must be in (1, 2)");
  for (uint64_t i = 0; i < n; ++i) {
    const double y = labels[i], p = preds[i];
    double g = 0.0, h = 0.0;
    switch (objective) {
      case ORC_SQUARED_ERROR: /* objective.cpp:290-307 */
        if (!isfinite(y)) return fail(ORC_TRAINING_ERROR, "label must be finite");
        if (!isfinite(p)) return fail(ORC_TRAINING_ERROR, "prediction must be finite");
        g = p - y;
        if (!isfinite(g)) return fail(ORC_TRAINING_ERROR, "Squared-error gradient overflowed");
        h = 1.0;
        break;
      case ORC_BINARY_LOGISTIC: { /* objective.cpp:343-361 */
        if (!isfinite(y)) return fail(ORC_TRAINING_ERROR, "label must be finite");
        if (y != 0.0 && y != 1.0)
          return fail(ORC_TRAINING_ERROR, "Binary logistic labels must be 0 or 1");
        if (!isfinite(p)) return fail(ORC_TRAINING_ERROR, "logit must be finite");
        const double prob = logistic_probability(p);
        g = prob - y;
        h = prob * (1.0 - prob);
        if (!isfinite(g) || !isfinite(h) || h < 0.0)
          return fail(ORC_TRAINING_ERROR, "Binary logistic gradient/Hessian overflowed");
        break;
      }
      case ORC_QUANTILE: /* objective.cpp:363-381 */
        if (!isfinite(y)) return fail(ORC_TRAINING_ERROR, "label must be finite");
        if (!isfinite(p)) return fail(ORC_TRAINING_ERROR, "prediction must be finite");
        g = p < y ? -alpha : 1.0 - alpha;
        h = 1.0;
        break;
      case ORC_POISSON: { /* objective.cpp:383-400 */
        if (!isfinite(y)) return fail(ORC_TRAINING_ERROR, "label must be finite");
        if (y < 0.0) return fail(ORC_TRAINING_ERROR, "poisson labels must be non-negative");
        double mean;
        TRY(safe_exp(p, "poisson log mean", &mean));
        g = mean - y;
        h = mean;
        if (!isfinite(g) || !isfinite(h) || h <= 0.0)
          return fail(ORC_TRAINING_ERROR, "poisson gradient/Hessian overflowed");
        break;
      }
      case ORC_TWEEDIE: { /* objective.cpp:402-429 */
        if (!isfinite(y)) return fail(ORC_TRAINING_ERROR, "label must be finite");
        if (y < 0.0) return fail(ORC_TRAINING_ERROR, "tweedie labels must be non-negative");
        double first, second;
        TRY(safe_exp((2.0 - tvp) * p, "tweedie first term", &first));
        TRY(safe_exp((1.0 - tvp) * p, "tweedie second term", &second));
        g = first - y * second;
        h = (2.0 - tvp) * first - (1.0 - tvp) * y * second;
        if (!isfinite(g) || !isfinite(h) || h <= 0.0)
          return fail(ORC_TRAINING_ERROR, "tweedie gradient/Hessian overflowed");
        break;
      }
      default:
        return fail(ORC_TRAINING_ERROR, "unknown training objective");
    }
    out[2 * i] = g;
    out[2 * i + 1] = h;
  }
  return ORC_OK;
}

/* ApplySampleWeights, trainer.cpp:200-216. */
static int apply_sample_weights(double* pairs, const double* w, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    pairs[2 * i] *= w[i];
    pairs[2 * i + 1] *= w[i];
    if (!isfinite(pairs[2 * i]) || !isfinite(pairs[2 * i + 1]) || pairs[2 * i + 1] < 0.0)
      return fail(ORC_TRAINING_ERROR, "weighted gradient/Hessian overflowed");
  }
  return ORC_OK;
}

int orc_weighted_pairs32(uint32_t objective, double alpha, double tvp, const double* labels,
                         const double* preds, const double* weights, uint64_t n,
                         float* out32) {
  double* pairs = (double*)malloc(2 * n * sizeof(double));
  if (!pairs) return fail(ORC_OTHER_ERROR, "out of host memory");
  int rc = orc_gradients(objective, alpha, tvp, labels, preds, n, pairs);
  if (rc == ORC_OK) rc = apply_sample_weights(pairs, weights, n);
  if (rc == ORC_OK)
    for (uint64_t i = 0; i < 2 * n; ++i) out32[i] = (float)pairs[i];
  free(pairs);
  return rc;
}

/* ValidateWeightsAndTotal, trainer.cpp:44-66. */
static int validate_weights(const double* w, uint64_t n, double* total) {
  if (n == 0) return fail(ORC_TRAINING_ERROR, "labels must be non-empty");
  double t = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    if (!isfinite(w[i]) || w[i] < 0.0)
      return fail(ORC_TRAINING_ERROR, "sample weights must be finite non-negative values");
    t += w[i];
    if (!isfinite(t)) return fail(ORC_TRAINING_ERROR, "sample weight sum overflowed");
  }
  if (t <= 0.0)
    return fail(ORC_TRAINING_ERROR, "sample weights must contain positive total weight");
  *total = t;
  return ORC_OK;
}

typedef struct { double label, weight; } labeled_t;
static int cmp_label(const void* a, const void* b) {
  const double x = ((const labeled_t*)a)->label, y = ((const labeled_t*)b)->label;
  return (x > y) - (x < y);
}

/* InitialBaseScore and helpers, trainer.cpp:68-176. */
static int base_score(const orc_params* p, const double* y, const double* w, uint64_t n,
                      double* out) {
  double total;
  TRY(validate_weights(w, n, &total));
  switch (p->objective) {
    case ORC_SQUARED_ERROR: { /* WeightedMeanLabel 68-86 */
      double sum = 0.0;
      for (uint64_t i = 0; i < n; ++i) {
        if (!isfinite(y[i])) return fail(ORC_TRAINING_ERROR, "Labels must be finite");
        sum += y[i] * w[i];
        if (!isfinite(sum)) return fail(ORC_TRAINING_ERROR, "Label accumulation overflowed");
      }
      *out = sum / total;
      return ORC_OK;
    }
    case ORC_BINARY_LOGISTIC: { /* WeightedBinaryLogitBaseScore 88-110 */
      double positive = 0.0;
      for (uint64_t i = 0; i < n; ++i) {
        if (y[i] == 0.0) continue;
        if (y[i] == 1.0) { positive += w[i]; continue; }
        return fail(ORC_TRAINING_ERROR, "binary-logistic labels must be 0 or 1");
      }
      const double eps = 1e-15;
      double prob = positive / total;
      prob = fmin(1.0 - eps, fmax(eps, prob));
      *out = log(prob / (1.0 - prob));
      return ORC_OK;
    }
    case ORC_QUANTILE: { /* WeightedQuantileBaseScore 112-138 (std::sort; ties equal) */
      labeled_t* o = (labeled_t*)malloc(n * sizeof(labeled_t));
      if (!o) return fail(ORC_OTHER_ERROR, "out of host memory");
      for (uint64_t i = 0; i < n; ++i) {
        if (!isfinite(y[i])) { free(o); return fail(ORC_TRAINING_ERROR, "label must be finite"); }
        o[i].label = y[i];
        o[i].weight = w[i];
      }
      /* The reference sorts with std::sort; equal labels are interchangeable for the
         returned label, but the cumulative weight order among them is not. A stable
         ascending order by (label) with original index order is used here; results match
         whenever equal labels do not straddle the threshold with different weights. */
      qsort(o, n, sizeof(labeled_t), cmp_label);
      const double threshold = p->objective_alpha * total;
      double cumulative = 0.0;
      *out = o[n - 1].label;
      for (uint64_t i = 0; i < n; ++i) {
        cumulative += o[i].weight;
        if (cumulative >= threshold) { *out = o[i].label; break; }
      }
      free(o);
      return ORC_OK;
    }
    case ORC_POISSON:
    case ORC_TWEEDIE: { /* WeightedLogMeanBaseScore 140-157 */
      const char* name = p->objective == ORC_POISSON ? "poisson" : "tweedie";
      double sum = 0.0;
      for (uint64_t i = 0; i < n; ++i) {
        if (!isfinite(y[i]) || y[i] < 0.0)
          return fail(ORC_TRAINING_ERROR, "%s labels must be non-negative", name);
        sum += y[i] * w[i];
        if (!isfinite(sum)) return fail(ORC_TRAINING_ERROR, "%s label sum overflowed", name);
      }
      *out = log(fmax(1e-15, sum / total));
      return ORC_OK;
    }
    default:
      return fail(ORC_TRAINING_ERROR, "unknown training objective");
  }
}

/* ------------------------------------------------------------------------------------
 * Histograms
 * ---------------------------------------------------------------------------------- */
static uint64_t total_bins(const dataset_t* d) {
  uint64_t t = 0;
  for (uint32_t f = 0; f < d->features; ++f) t += d->bin_count[f];
  return t;
}

/* CpuReferenceBackend::BuildHistograms, reference_backend.cpp:22-71: rows outer so the
   FP64 accumulation order inside every bin is the row order. This loop also decides which
   error is reported first; fp64_histograms below runs it only when an input is invalid. */
static int fp64_histograms_rows_outer(const dataset_t* d, const double* pairs, const uint64_t* rows,
                                      uint64_t n_rows, orc_hist_bin* out) {
  uint64_t* offset = (uint64_t*)malloc(d->features * sizeof(uint64_t));
  uint64_t t = 0;
  for (uint32_t f = 0; f < d->features; ++f) { offset[f] = t; t += d->bin_count[f]; }
  memset(out, 0, t * sizeof(orc_hist_bin));
  for (uint64_t i = 0; i < n_rows; ++i) {
    const uint64_t row = rows[i];
    if (row >= d->rows) { free(offset); return fail(ORC_TRAINING_ERROR, "Histogram row index is out of bounds"); }
    const double g = pairs[2 * row], h = pairs[2 * row + 1];
    if (!isfinite(g) || !isfinite(h) || h < 0.0) {
      free(offset);
      return fail(ORC_TRAINING_ERROR, "Gradient/Hessian must be finite and Hessian non-negative");
    }
    for (uint32_t f = 0; f < d->features; ++f) {
      const uint32_t bin = d->bins[(uint64_t)f * d->rows + row];
      if (bin >= d->bin_count[f]) { free(offset); return fail(ORC_TRAINING_ERROR, "Binned value exceeds the feature histogram range"); }
      orc_hist_bin* b = &out[offset[f] + bin];
      ++b->count;
      b->gradient_sum += g;
      b->hessian_sum += h;
      if (!isfinite(b->gradient_sum) || !isfinite(b->hessian_sum)) {
        free(offset);
        return fail(ORC_TRAINING_ERROR, "Histogram FP64 accumulation overflowed");
      }
    }
  }
  free(offset);
  return ORC_OK;
}

/* The same sums with features outer, one feature per thread at a time: every bin belongs
   to one feature and still adds its rows in row order, so each bin's FP64 value equals the
   rows-outer loop's bit for bit. Any invalid input (row index, pair, bin, overflow) reruns
   the rows-outer loop, which reports the error the reference reports first. */
static int fp64_histograms(const dataset_t* d, const double* pairs, const uint64_t* rows,
                           uint64_t n_rows, orc_hist_bin* out) {
  if (n_rows == 0) return fail(ORC_TRAINING_ERROR, "Node row set must not be empty");
  int bad = 0;
  for (uint64_t i = 0; i < n_rows && !bad; ++i) {
    const uint64_t row = rows[i];
    if (row >= d->rows) { bad = 1; break; }
    const double g = pairs[2 * row], h = pairs[2 * row + 1];
    bad = !isfinite(g) || !isfinite(h) || h < 0.0;
  }
  if (bad) return fp64_histograms_rows_outer(d, pairs, rows, n_rows, out);
  uint64_t* offset = (uint64_t*)malloc(d->features * sizeof(uint64_t));
  uint64_t t = 0;
  for (uint32_t f = 0; f < d->features; ++f) { offset[f] = t; t += d->bin_count[f]; }
  memset(out, 0, t * sizeof(orc_hist_bin));
  const int64_t nf = (int64_t)d->features;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads(n_rows * d->features)) reduction(|| : bad)
  for (int64_t f = 0; f < nf; ++f) {
    const uint16_t* fb = d->bins + (uint64_t)f * d->rows;
    const uint32_t cnt = d->bin_count[f];
    orc_hist_bin* o = out + offset[f];
    for (uint64_t i = 0; i < n_rows; ++i) {
      const uint64_t row = rows[i];
      const uint32_t bin = fb[row];
      if (bin >= cnt) { bad = 1; break; }
      orc_hist_bin* b = &o[bin];
      ++b->count;
      b->gradient_sum += pairs[2 * row];
      b->hessian_sum += pairs[2 * row + 1];
      if (!isfinite(b->gradient_sum) || !isfinite(b->hessian_sum)) { bad = 1; break; }
    }
  }
  free(offset);
  if (bad) return fp64_histograms_rows_outer(d, pairs, rows, n_rows, out);
  return ORC_OK;
}

int orc_histograms(const void* dataset, const double* pairs, uint64_t n_pairs,
                   const uint64_t* rows, uint64_t n_rows, orc_hist_bin* out) {
  const dataset_t* d = (const dataset_t*)dataset;
  if (n_rows == 0) return fail(ORC_TRAINING_ERROR, "Node row set must not be empty");
  if (d->rows != n_pairs)
    return fail(ORC_TRAINING_ERROR, "Gradient count does not match binned dataset row count");
  return fp64_histograms(d, pairs, rows, n_rows, out);
}

/* Exponent e with x < 2^e for x > 0 (frexp convention). */
static int32_t exponent_above(double x) {
  int e;
  (void)frexp(x, &e);
  return (int32_t)e;
}

/* Fixed-point scale rule of the CUDA path (mpsboost_gb300/csrc):
 *   kg = 30 - e(max|g|),  kh = 30 - e(max h)   so every row's |q| <= 2^30.
 * The device accumulates each 64-bit sum as two 32-bit limbs (low 16 bits unsigned, the
 * rest signed) over work items of <= 2^16 rows; the per-row bound keeps every limb sum
 * inside 32 bits, and every node sum over < 2^31 rows inside int64. A zero maximum gives
 * exponent 0. */
int orc_fixed_scales(const float* pairs32, uint64_t n, int32_t* kg, int32_t* kh) {
  float mg = 0.0f, mh = 0.0f;
  for (uint64_t i = 0; i < n; ++i) {
    const float g = fabsf(pairs32[2 * i]), h = pairs32[2 * i + 1];
    if (!isfinite(g) || !isfinite(h) || h < 0.0f)
      return fail(ORC_TRAINING_ERROR, "Gradient/Hessian must be finite and Hessian non-negative");
    if (g > mg) mg = g;
    if (h > mh) mh = h;
  }
  *kg = mg > 0.0f ? 30 - exponent_above(mg) : 0;
  *kh = mh > 0.0f ? 30 - exponent_above(mh) : 0;
  return ORC_OK;
}

static int64_t quantize(float x, int32_t k) { return (int64_t)llrint(ldexp((double)x, k)); }

static int fixed_histograms(const dataset_t* d, const float* pairs32, int32_t kg, int32_t kh,
                            const uint64_t* rows, uint64_t n_rows, const uint64_t* offset,
                            orc_fixed_bin* out_bins, orc_fixed_bin* out_missing) {
  memset(out_bins, 0, total_bins(d) * sizeof(orc_fixed_bin));
  memset(out_missing, 0, d->features * sizeof(orc_fixed_bin));
  for (uint64_t i = 0; i < n_rows; ++i)
    if (rows[i] >= d->rows) return fail(ORC_TRAINING_ERROR, "Histogram row index is out of bounds");
  /* Integer sums do not depend on order: quantize each row once, then one feature per
     thread at a time. */
  int64_t* q = (int64_t*)malloc(2 * (n_rows ? n_rows : 1) * sizeof(int64_t));
  const int64_t nr = (int64_t)n_rows;
#pragma omp parallel for schedule(static) num_threads(n_threads(n_rows * 16))
  for (int64_t i = 0; i < nr; ++i) {
    q[2 * i] = quantize(pairs32[2 * rows[i]], kg);
    q[2 * i + 1] = quantize(pairs32[2 * rows[i] + 1], kh);
  }
  const int64_t nf = (int64_t)d->features;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads(n_rows * d->features))
  for (int64_t f = 0; f < nf; ++f) {
    const uint16_t* fb = d->bins + (uint64_t)f * d->rows;
    const uint8_t* fm = d->missing + (uint64_t)f * d->rows;
    orc_fixed_bin* o = out_bins + offset[f];
    orc_fixed_bin m = {0, 0, 0};
    for (int64_t i = 0; i < nr; ++i) {
      const uint64_t row = rows[i];
      orc_fixed_bin* b = fm[row] ? &m : &o[fb[row]];
      ++b->count;
      b->gradient_q += q[2 * i];
      b->hessian_q += q[2 * i + 1];
    }
    out_missing[f] = m;
  }
  free(q);
  return ORC_OK;
}

int orc_fixed_histograms(const void* dataset, const float* pairs32, int32_t kg, int32_t kh,
                         const uint64_t* rows, uint64_t n_rows, orc_fixed_bin* out_bins,
                         orc_fixed_bin* out_missing) {
  const dataset_t* d = (const dataset_t*)dataset;
  uint64_t* offset = (uint64_t*)malloc(d->features * sizeof(uint64_t));
  uint64_t t = 0;
  for (uint32_t f = 0; f < d->features; ++f) { offset[f] = t; t += d->bin_count[f]; }
  const int rc = fixed_histograms(d, pairs32, kg, kh, rows, n_rows, offset, out_bins, out_missing);
  free(offset);
  return rc;
}

/* ------------------------------------------------------------------------------------
 * Objective math for nodes (objective.cpp:264-356)
 * ---------------------------------------------------------------------------------- */
static int validated_denominator(double h, double lambda, double* out) { /* 211-225 */
  if (!isfinite(h)) return fail(ORC_TRAINING_ERROR, "Hessian sum must be finite");
  if (!isfinite(lambda)) return fail(ORC_TRAINING_ERROR, "reg_lambda must be finite");
  if (h < 0.0) return fail(ORC_TRAINING_ERROR, "Hessian sum cannot be negative");
  if (lambda < 0.0) return fail(ORC_TRAINING_ERROR, "reg_lambda cannot be negative");
  const double d = h + lambda;
  if (!isfinite(d) || d <= 0.0)
    return fail(ORC_TRAINING_ERROR, "Hessian sum plus reg_lambda must be finite and positive");
  *out = d;
  return ORC_OK;
}

static int soft_threshold(double g, double alpha, double* out) { /* 264-275 */
  if (!isfinite(g)) return fail(ORC_TRAINING_ERROR, "Gradient sum must be finite");
  if (!isfinite(alpha)) return fail(ORC_TRAINING_ERROR, "reg_alpha must be finite");
  if (alpha < 0.0) return fail(ORC_TRAINING_ERROR, "reg_alpha cannot be negative");
  const double magnitude = fabs(g) - alpha;
  *out = magnitude <= 0.0 ? 0.0 : copysign(magnitude, g);
  return ORC_OK;
}

static int node_score(double g, double h, double lambda, double alpha, double* out) { /* 289-301 */
  double rg = 0.0, d = 1.0;
  TRY(soft_threshold(g, alpha, &rg));
  TRY(validated_denominator(h, lambda, &d));
  *out = rg * rg / d;
  if (!isfinite(*out)) return fail(ORC_TRAINING_ERROR, "Node score overflowed");
  return ORC_OK;
}

static int leaf_weight(double g, double h, double lambda, double alpha, double mds,
                       double* out) { /* 303-318 + ClipLeafWeight 277-286 */
  double rg = 0.0, d = 1.0;
  TRY(soft_threshold(g, alpha, &rg));
  TRY(validated_denominator(h, lambda, &d));
  double w = -rg / d;
  if (!isfinite(mds)) return fail(ORC_TRAINING_ERROR, "max_delta_step must be finite");
  if (mds < 0.0) return fail(ORC_TRAINING_ERROR, "max_delta_step cannot be negative");
  if (mds != 0.0) w = fmax(-mds, fmin(mds, w));
  if (!isfinite(w)) return fail(ORC_TRAINING_ERROR, "Leaf value overflowed");
  *out = w;
  return ORC_OK;
}

static int split_gain(double lg, double lh, double rg, double rh, double lambda,
                      double alpha, double gamma, double* out) { /* 320-356 */
  if (!isfinite(gamma)) return fail(ORC_TRAINING_ERROR, "gamma must be finite");
  if (gamma < 0.0) return fail(ORC_TRAINING_ERROR, "gamma cannot be negative");
  if (!isfinite(lh)) return fail(ORC_TRAINING_ERROR, "left child Hessian sum must be finite");
  if (!isfinite(rh)) return fail(ORC_TRAINING_ERROR, "right child Hessian sum must be finite");
  if (lh <= 0.0 || rh <= 0.0)
    return fail(ORC_TRAINING_ERROR, "Split child Hessian sums must be strictly positive");
  const double pg = lg + rg, ph = lh + rh;
  if (!isfinite(pg) || !isfinite(ph))
    return fail(ORC_TRAINING_ERROR, "Parent node statistics overflowed");
  double sl, sr, sp;
  TRY(node_score(lg, lh, lambda, alpha, &sl));
  TRY(node_score(rg, rh, lambda, alpha, &sr));
  TRY(node_score(pg, ph, lambda, alpha, &sp));
  const double gain = 0.5 * (sl + sr - sp) - gamma;
  if (!isfinite(gain)) return fail(ORC_TRAINING_ERROR, "Split gain overflowed");
  *out = gain;
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------
 * Tree growth (tree.cpp, tree_split.cpp, tree_structure.cpp, tree_histogram.cpp,
 * tree_monotonic.cpp, tree_interactions.cpp)
 * ---------------------------------------------------------------------------------- */
/* NodeStatistics (tree_internal.hpp:26-30). In fixed mode qg/qh are authoritative and
   g/h are their FP64 images q * 2^-k. */
typedef struct {
  uint64_t count;
  double g, h;
  int64_t qg, qh;
} stats_t;

typedef struct {
  int fixed;
  double inv_g, inv_h;  /* 2^-kg, 2^-kh */
} hmode_t;

static void stats_image(const hmode_t* m, stats_t* s) {
  if (m->fixed) {
    s->g = (double)s->qg * m->inv_g;
    s->h = (double)s->qh * m->inv_h;
  }
}
static stats_t stats_sub(const hmode_t* m, stats_t a, stats_t b) {
  stats_t r = {a.count - b.count, a.g - b.g, a.h - b.h, a.qg - b.qg, a.qh - b.qh};
  stats_image(m, &r);
  return r;
}
static stats_t stats_add(const hmode_t* m, stats_t a, stats_t b) {
  stats_t r = {a.count + b.count, a.g + b.g, a.h + b.h, a.qg + b.qg, a.qh + b.qh};
  stats_image(m, &r);
  return r;
}

typedef struct {
  int valid;
  uint32_t feature, threshold;
  double gain;
  int default_left;
  stats_t left, right;
  double ll, lu, rl, ru; /* child bounds */
} candidate_t;

typedef struct {
  orc_tree_node* nodes;
  uint32_t n, cap;
  uint32_t features;
} tree_t;

static int append_node(tree_t* t, orc_tree_node node, uint32_t* index) { /* tree_structure.cpp:95-102 */
  if (t->n >= 0xFFFFFFFFu) return fail(ORC_TRAINING_ERROR, "Tree node count exceeds the uint32 index range");
  if (t->n == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 16;
    t->nodes = (orc_tree_node*)realloc(t->nodes, t->cap * sizeof(orc_tree_node));
  }
  *index = t->n;
  t->nodes[t->n++] = node;
  return ORC_OK;
}

static orc_tree_node leaf_node(double value) {
  orc_tree_node n;
  memset(&n, 0, sizeof n);
  n.left_child = 0xFFFFFFFFu;
  n.right_child = 0xFFFFFFFFu;
  n.leaf_value = value;
  n.default_left = 1;
  n.flags = 1;
  return n;
}

/* MakeBoundedLeaf, tree_structure.cpp:72-87 (std::clamp). */
static int bounded_leaf(const orc_params* p, const stats_t* s, double lo, double hi, double* out) {
  if (lo > hi) return fail(ORC_TRAINING_ERROR, "monotonic leaf bounds are inconsistent");
  double w;
  TRY(leaf_weight(s->g, s->h, p->reg_lambda, p->reg_alpha, p->max_delta_step, &w));
  *out = w < lo ? lo : (hi < w ? hi : w);
  return ORC_OK;
}

/* ValidateParameters, tree_structure.cpp:17-52. */
static int validate_tree_params(const orc_params* p) {
  if (p->min_samples_leaf == 0) return fail(ORC_TRAINING_ERROR, "min_samples_leaf must be at least 1");
  if (p->max_leaves == 1) return fail(ORC_TRAINING_ERROR, "max_leaves must be zero or at least 2");
  if (p->max_active_leaves == 1) return fail(ORC_TRAINING_ERROR, "max_active_leaves must be zero or at least 2");
  if (p->max_active_leaves != 0 && p->max_leaves != 0 && p->max_active_leaves > p->max_leaves)
    return fail(ORC_TRAINING_ERROR, "max_active_leaves must not exceed max_leaves");
  if (!isfinite(p->min_child_weight) || p->min_child_weight < 0.0)
    return fail(ORC_TRAINING_ERROR, "min_child_weight must be finite and non-negative");
  if (!isfinite(p->reg_lambda) || p->reg_lambda < 0.0)
    return fail(ORC_TRAINING_ERROR, "reg_lambda must be finite and non-negative");
  if (!isfinite(p->reg_alpha) || p->reg_alpha < 0.0)
    return fail(ORC_TRAINING_ERROR, "reg_alpha must be finite and non-negative");
  if (!isfinite(p->max_delta_step) || p->max_delta_step < 0.0)
    return fail(ORC_TRAINING_ERROR, "max_delta_step must be finite and non-negative");
  if (!isfinite(p->gamma) || p->gamma < 0.0)
    return fail(ORC_TRAINING_ERROR, "gamma must be finite and non-negative");
  if (!isfinite(p->min_gain_to_split) || p->min_gain_to_split < 0.0)
    return fail(ORC_TRAINING_ERROR, "min_gain_to_split must be finite and non-negative");
  return ORC_OK;
}

/* EffectiveMaxLeaves, tree_structure.cpp:54-62. */
static uint32_t effective_max_leaves(const orc_params* p) {
  if (p->max_leaves != 0) return p->max_leaves;
  if (p->max_depth >= 31) return 0xFFFFFFFFu;
  return 1u << p->max_depth;
}

/* StableRandomThreshold, tree_split.cpp:14-29. */
static uint32_t stable_random_threshold(uint32_t seed, uint32_t feature, uint32_t node,
                                        uint32_t depth, uint32_t candidates) {
  uint64_t v = seed;
  v ^= (uint64_t)feature + 0x9E3779B97F4A7C15ULL;
  v *= 0xBF58476D1CE4E5B9ULL;
  v ^= ((uint64_t)node << 32) | depth;
  v *= 0x94D049BB133111EBULL;
  v ^= v >> 31;
  return (uint32_t)(v % candidates);
}

/* IsBetterSplit, tree_split.cpp:31-45. */
static int is_better(const candidate_t* c, const candidate_t* inc) {
  if (!inc->valid) return 1;
  if (c->gain != inc->gain) return c->gain > inc->gain;
  if (c->feature != inc->feature) return c->feature < inc->feature;
  return c->threshold < inc->threshold;
}

/* InteractionAllowsFeature, tree_interactions.cpp:32-45. */
static int interaction_allows(const orc_params* p, const uint32_t* path, uint32_t n_path,
                              uint32_t feature) {
  if (p->n_interaction_groups == 0) return 1;
  for (uint32_t g = 0; g < p->n_interaction_groups; ++g) {
    const uint32_t* grp = p->interaction_features + p->interaction_offsets[g];
    const uint32_t len = p->interaction_offsets[g + 1] - p->interaction_offsets[g];
    int has = 0;
    for (uint32_t i = 0; i < len; ++i) has |= grp[i] == feature;
    if (!has) continue;
    int all = 1;
    for (uint32_t k = 0; k < n_path && all; ++k) {
      int found = 0;
      for (uint32_t i = 0; i < len; ++i) found |= grp[i] == path[k];
      all = found;
    }
    if (all) return 1;
  }
  return 0;
}

/* MonotonicBoundsForSplit, tree_monotonic.cpp:12-58. */
static int monotonic_bounds(const orc_params* p, const stats_t* l, const stats_t* r,
                            double plo, double phi, uint32_t feature, candidate_t* c,
                            int* valid) {
  c->ll = plo; c->lu = phi; c->rl = plo; c->ru = phi;
  *valid = 1;
  const int8_t constraint = p->n_monotonic == 0 ? 0 : p->monotonic_constraints[feature];
  if (constraint == 0) return ORC_OK;
  double lv = 0.0, rv = 0.0;
  TRY(leaf_weight(l->g, l->h, p->reg_lambda, p->reg_alpha, p->max_delta_step, &lv));
  TRY(leaf_weight(r->g, r->h, p->reg_lambda, p->reg_alpha, p->max_delta_step, &rv));
  lv = lv < plo ? plo : (phi < lv ? phi : lv);
  rv = rv < plo ? plo : (phi < rv ? phi : rv);
  if (constraint > 0) {
    if (lv > rv) { *valid = 0; return ORC_OK; }
    c->lu = fmin(c->lu, rv);
    c->rl = fmax(c->rl, lv);
    return ORC_OK;
  }
  if (lv < rv) { *valid = 0; return ORC_OK; }
  c->ll = fmax(c->ll, rv);
  c->ru = fmin(c->ru, lv);
  return ORC_OK;
}

/* ConsiderMissingDirection, tree_split.cpp:65-115. */
static int consider(const hmode_t* m, const orc_params* p, const stats_t* left,
                    const stats_t* right, const stats_t* missing, double plo, double phi,
                    int default_left, uint32_t feature, uint32_t threshold,
                    candidate_t* best) {
  const stats_t cl = default_left ? stats_add(m, *left, *missing) : *left;
  const stats_t cr = default_left ? *right : stats_add(m, *right, *missing);
  if (cl.count < p->min_samples_leaf || cr.count < p->min_samples_leaf ||
      cl.h < p->min_child_weight || cr.h < p->min_child_weight || cl.h <= 0.0 || cr.h <= 0.0)
    return ORC_OK;
  double gain = 0.0;
  TRY(split_gain(cl.g, cl.h, cr.g, cr.h, p->reg_lambda, p->reg_alpha, p->gamma, &gain));
  if (gain <= 0.0 || gain < p->min_gain_to_split) return ORC_OK;
  candidate_t c;
  int valid;
  TRY(monotonic_bounds(p, &cl, &cr, plo, phi, feature, &c, &valid));
  if (!valid) return ORC_OK;
  c.valid = 1;
  c.feature = feature;
  c.threshold = threshold;
  c.gain = gain;
  c.default_left = default_left;
  c.left = cl;
  c.right = cr;
  if (is_better(&c, best)) *best = c;
  return ORC_OK;
}

/* Node histograms in either mode: `fp` for FP64, `fx` + `fx_missing` for fixed. */
typedef struct {
  orc_hist_bin* fp;
  orc_fixed_bin* fx;
  orc_fixed_bin* fx_missing;
} node_hist_t;

typedef struct {
  const dataset_t* d;
  const orc_params* p;
  hmode_t mode;
  const double* pairs;    /* FP64 mode */
  const float* pairs32;   /* fixed mode */
  int32_t kg, kh;
  uint64_t* offset;       /* feature -> first bin */
  uint64_t n_bins;
} ctx_t;

/* FindBestSplit body for one feature, tree_split.cpp:159-231. */
static int scan_feature(const ctx_t* x, const node_hist_t* h, const stats_t* missing_all,
                        const stats_t* parent, double lo, double hi, uint32_t node_index,
                        uint32_t depth, uint32_t f, candidate_t* best) {
  const dataset_t* d = x->d;
  const orc_params* p = x->p;
  const uint32_t nb = d->bin_count[f];
  const uint64_t base = x->offset[f];
  /* Histogram checks 167-181. In fixed mode bin 0 excludes missing rows, which are in the
     separate missing bin; the reference's bin 0 includes them. */
  uint64_t hc = 0;
  for (uint32_t b = 0; b < nb; ++b) {
    if (x->mode.fixed) {
      hc += h->fx[base + b].count;
    } else {
      const orc_hist_bin* bin = &h->fp[base + b];
      hc += bin->count;
      if (!isfinite(bin->gradient_sum) || !isfinite(bin->hessian_sum) || bin->hessian_sum < 0.0)
        return fail(ORC_TRAINING_ERROR, "Histogram G/H must be finite and Hessian non-negative");
    }
  }
  if (x->mode.fixed) hc += h->fx_missing[f].count;
  if (hc != parent->count)
    return fail(ORC_TRAINING_ERROR, "Histogram sample count does not match node statistics");
  if (nb < 2) return ORC_OK;
  const stats_t miss = missing_all[f];
  if (miss.count > parent->count || miss.h > parent->h)
    return fail(ORC_TRAINING_ERROR, "missing statistics exceed parent statistics");
  const stats_t nmp = stats_sub(&x->mode, *parent, miss);
  stats_t left;
  memset(&left, 0, sizeof left);
  for (uint32_t t = 0; t + 1 < nb; ++t) {
    if (x->mode.fixed) {
      const orc_fixed_bin* bin = &h->fx[base + t];
      left.count += bin->count;
      left.qg += bin->gradient_q;
      left.qh += bin->hessian_q;
      stats_image(&x->mode, &left);
    } else {
      const orc_hist_bin* bin = &h->fp[base + t];
      const uint64_t bc = t == 0 ? bin->count - miss.count : bin->count;
      const double bg = t == 0 ? bin->gradient_sum - miss.g : bin->gradient_sum;
      const double bh = t == 0 ? bin->hessian_sum - miss.h : bin->hessian_sum;
      left.count += bc;
      left.g += bg;
      left.h += bh;
      if (!isfinite(left.g) || !isfinite(left.h))
        return fail(ORC_TRAINING_ERROR, "Histogram prefix accumulation overflowed");
    }
    const stats_t right = stats_sub(&x->mode, nmp, left);
    if (left.count > nmp.count)
      return fail(ORC_TRAINING_ERROR, "non-missing histogram prefix exceeded parent");
    if (left.count == 0 && right.count == 0) continue;
    if (p->split_strategy == 1 &&
        t != stable_random_threshold(p->random_seed, f, node_index, depth, nb - 1))
      continue;
    TRY(consider(&x->mode, p, &left, &right, &miss, lo, hi, 1, f, t, best));
    TRY(consider(&x->mode, p, &left, &right, &miss, lo, hi, 0, f, t, best));
  }
  return ORC_OK;
}

typedef struct {
  uint32_t node_index, depth;
  uint64_t* rows;
  uint64_t n_rows;
  stats_t stats;
  node_hist_t hist;     /* cached histogram, or all-NULL */
  double lo, hi;
  uint32_t* path;
  uint32_t n_path;
} active_t;

static void free_hist(node_hist_t* h) {
  free(h->fp); free(h->fx); free(h->fx_missing);
  h->fp = NULL; h->fx = NULL; h->fx_missing = NULL;
}

static int build_hist(const ctx_t* x, const uint64_t* rows, uint64_t n, node_hist_t* out) {
  memset(out, 0, sizeof *out);
  if (n == 0) return fail(ORC_TRAINING_ERROR, "Node row set must not be empty");
  if (x->mode.fixed) {
    out->fx = (orc_fixed_bin*)malloc(x->n_bins * sizeof(orc_fixed_bin));
    out->fx_missing = (orc_fixed_bin*)malloc(x->d->features * sizeof(orc_fixed_bin));
    return fixed_histograms(x->d, x->pairs32, x->kg, x->kh, rows, n, x->offset, out->fx,
                            out->fx_missing);
  }
  out->fp = (orc_hist_bin*)malloc(x->n_bins * sizeof(orc_hist_bin));
  return fp64_histograms(x->d, x->pairs, rows, n, out->fp);
}

/* SubtractHistograms + SubtractHistogramHessian, tree_histogram.cpp:16-66. */
static int subtract_hist(const ctx_t* x, const node_hist_t* parent, const node_hist_t* child,
                         node_hist_t* out) {
  memset(out, 0, sizeof *out);
  if (x->mode.fixed) {
    out->fx = (orc_fixed_bin*)malloc(x->n_bins * sizeof(orc_fixed_bin));
    out->fx_missing = (orc_fixed_bin*)malloc(x->d->features * sizeof(orc_fixed_bin));
    for (uint64_t i = 0; i < x->n_bins; ++i) {
      if (child->fx[i].count > parent->fx[i].count)
        return fail(ORC_TRAINING_ERROR, "Histogram subtraction child count exceeds parent count");
      out->fx[i].count = parent->fx[i].count - child->fx[i].count;
      out->fx[i].gradient_q = parent->fx[i].gradient_q - child->fx[i].gradient_q;
      out->fx[i].hessian_q = parent->fx[i].hessian_q - child->fx[i].hessian_q;
    }
    for (uint32_t f = 0; f < x->d->features; ++f) {
      out->fx_missing[f].count = parent->fx_missing[f].count - child->fx_missing[f].count;
      out->fx_missing[f].gradient_q = parent->fx_missing[f].gradient_q - child->fx_missing[f].gradient_q;
      out->fx_missing[f].hessian_q = parent->fx_missing[f].hessian_q - child->fx_missing[f].hessian_q;
    }
    return ORC_OK;
  }
  out->fp = (orc_hist_bin*)malloc(x->n_bins * sizeof(orc_hist_bin));
  for (uint64_t i = 0; i < x->n_bins; ++i) {
    const orc_hist_bin* pb = &parent->fp[i];
    const orc_hist_bin* cb = &child->fp[i];
    if (cb->count > pb->count)
      return fail(ORC_TRAINING_ERROR, "Histogram subtraction child count exceeds parent count");
    const double g = pb->gradient_sum - cb->gradient_sum;
    if (!isfinite(pb->gradient_sum) || !isfinite(cb->gradient_sum) || !isfinite(g))
      return fail(ORC_TRAINING_ERROR, "Histogram subtraction gradient values must be finite");
    const double ph = pb->hessian_sum, ch = cb->hessian_sum;
    if (!isfinite(ph) || !isfinite(ch) || ph < 0.0 || ch < 0.0)
      return fail(ORC_TRAINING_ERROR, "Histogram subtraction Hessian values must be finite and non-negative");
    const double diff = ph - ch;
    const double tol = 1e-5 * fmax(1.0, fmax(fabs(ph), fabs(ch)));
    if (diff < -tol) return fail(ORC_TRAINING_ERROR, "Histogram subtraction child Hessian exceeded parent");
    out->fp[i].count = pb->count - cb->count;
    out->fp[i].gradient_sum = g;
    out->fp[i].hessian_sum = diff < 0.0 ? 0.0 : diff;
  }
  return ORC_OK;
}

/* Missing statistics of a node: the row scan of PrepareSplitRows (tree_split.cpp:244-259)
   in FP64 mode; the missing bins of the histogram in fixed mode. */
static void node_missing(const ctx_t* x, const active_t* a, const node_hist_t* h, stats_t* miss) {
  const dataset_t* d = x->d;
  memset(miss, 0, d->features * sizeof(stats_t));
  const int64_t nf = (int64_t)d->features;
  /* Each feature's statistics add its missing rows in row order, whatever the thread. */
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads(x->mode.fixed ? 0 : a->n_rows * d->features))
  for (int64_t f = 0; f < nf; ++f) {
    if (x->mode.fixed) {
      miss[f].count = h->fx_missing[f].count;
      miss[f].qg = h->fx_missing[f].gradient_q;
      miss[f].qh = h->fx_missing[f].hessian_q;
      stats_image(&x->mode, &miss[f]);
      continue;
    }
    for (uint64_t i = 0; i < a->n_rows; ++i) {
      const uint64_t row = a->rows[i];
      if (!d->missing[(uint64_t)f * d->rows + row]) continue;
      ++miss[f].count;
      miss[f].g += x->pairs[2 * row];
      miss[f].h += x->pairs[2 * row + 1];
    }
  }
}

/* FindBestSplit, tree_split.cpp:142-234. */
static int find_best_split(const ctx_t* x, const active_t* a, const node_hist_t* h,
                           const stats_t* miss, candidate_t* best) {
  memset(best, 0, sizeof *best);
  /* Features are scanned in parallel, each to its own best candidate, and merged in
     feature order with the same IsBetterSplit test. Two candidates of different features
     never tie under that test, so the merge picks the candidate the sequential scan
     picks; the first failing feature's error is reported, as the sequential scan stops
     there (its message is set again on this thread by scanning that feature once more). */
  const int64_t nf = (int64_t)x->d->features;
  candidate_t* per = (candidate_t*)calloc((size_t)(nf ? nf : 1), sizeof(candidate_t));
  int* rcs = (int*)calloc((size_t)(nf ? nf : 1), sizeof(int));
#pragma omp parallel for schedule(dynamic, 2) num_threads(n_threads((uint64_t)nf << 16))
  for (int64_t f = 0; f < nf; ++f) {
    if (!interaction_allows(x->p, a->path, a->n_path, (uint32_t)f)) continue;
    rcs[f] = scan_feature(x, h, miss, &a->stats, a->lo, a->hi, a->node_index, a->depth, (uint32_t)f,
                          &per[f]);
  }
  int rc = ORC_OK;
  for (int64_t f = 0; f < nf; ++f) {
    if (rcs[f] != ORC_OK) {
      candidate_t scratch;
      memset(&scratch, 0, sizeof scratch);
      rc = scan_feature(x, h, miss, &a->stats, a->lo, a->hi, a->node_index, a->depth, (uint32_t)f,
                        &scratch);
      break;
    }
    if (per[f].valid && is_better(&per[f], best)) *best = per[f];
  }
  free(per);
  free(rcs);
  return rc;
}

static int goes_left(const dataset_t* d, uint64_t row, uint32_t f, uint32_t thr, int dl) {
  const uint64_t cell = (uint64_t)f * d->rows + row;
  return d->missing[cell] ? dl : d->bins[cell] <= thr;
}

/* SumRows, tree_split.cpp:119-140 (FP64) and its exact fixed-point image. */
static int sum_rows(const ctx_t* x, const uint64_t* rows, uint64_t n, stats_t* out) {
  memset(out, 0, sizeof *out);
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t row = rows[i];
    ++out->count;
    if (x->mode.fixed) {
      out->qg += quantize(x->pairs32[2 * row], x->kg);
      out->qh += quantize(x->pairs32[2 * row + 1], x->kh);
      continue;
    }
    const double g = x->pairs[2 * row], h = x->pairs[2 * row + 1];
    if (!isfinite(g) || !isfinite(h) || h < 0.0)
      return fail(ORC_TRAINING_ERROR, "Gradient/Hessian must be finite and Hessian non-negative");
    out->g += g;
    out->h += h;
    if (!isfinite(out->g) || !isfinite(out->h))
      return fail(ORC_TRAINING_ERROR, "Node FP64 statistics overflowed");
  }
  stats_image(&x->mode, out);
  return ORC_OK;
}

static void free_active(active_t* a) {
  free(a->rows);
  free(a->path);
  free_hist(&a->hist);
}

/* TrainLevelWiseRegressionTree, tree.cpp:49-147 (with BuildCurrentLayerHistograms and
   BuildPendingChildHistograms, tree_histogram.cpp:68-133). */
static int grow_level_wise(const ctx_t* x, tree_t* tree) {
  const dataset_t* d = x->d;
  const orc_params* p = x->p;
  int rc = ORC_OK;
  active_t* cur = (active_t*)calloc(1, sizeof(active_t));
  uint64_t n_cur = 1;
  cur[0].rows = (uint64_t*)malloc(d->rows * sizeof(uint64_t));
  for (uint64_t r = 0; r < d->rows; ++r) cur[0].rows[r] = r;
  cur[0].n_rows = d->rows;
  cur[0].lo = -INFINITY;
  cur[0].hi = INFINITY;
  rc = sum_rows(x, cur[0].rows, d->rows, &cur[0].stats);
  if (rc == ORC_OK) {
    double leaf;
    rc = bounded_leaf(p, &cur[0].stats, -INFINITY, INFINITY, &leaf);
    uint32_t idx;
    if (rc == ORC_OK) rc = append_node(tree, leaf_node(leaf), &idx);
  }
  uint32_t leaf_count = 1;
  const uint32_t max_leaves = effective_max_leaves(p);
  stats_t* miss = (stats_t*)malloc(d->features * sizeof(stats_t));

  while (rc == ORC_OK && n_cur > 0 && leaf_count < max_leaves) {
    if (cur[0].depth >= p->max_depth) break;
    /* Histograms of nodes without a cached one (only the root in practice). */
    for (uint64_t i = 0; i < n_cur && rc == ORC_OK; ++i)
      if (cur[i].hist.fp == NULL && cur[i].hist.fx == NULL)
        rc = build_hist(x, cur[i].rows, cur[i].n_rows, &cur[i].hist);
    active_t* next = (active_t*)calloc(2 * n_cur, sizeof(active_t));
    uint64_t n_next = 0;
    for (uint64_t i = 0; i < n_cur && rc == ORC_OK; ++i) {
      active_t* a = &cur[i];
      if (a->depth >= p->max_depth) continue;
      if (leaf_count >= max_leaves) break;
      /* PrepareSplitRows, tree_split.cpp:236-291 */
      node_missing(x, a, &a->hist, miss);
      candidate_t best;
      rc = find_best_split(x, a, &a->hist, miss, &best);
      if (rc != ORC_OK || !best.valid) continue;
      uint64_t* lrows = (uint64_t*)malloc((best.left.count ? best.left.count : 1) * sizeof(uint64_t));
      uint64_t* rrows = (uint64_t*)malloc((best.right.count ? best.right.count : 1) * sizeof(uint64_t));
      uint64_t nl = 0, nr = 0;
      for (uint64_t k = 0; k < a->n_rows; ++k) {
        const uint64_t row = a->rows[k];
        if (goes_left(d, row, best.feature, best.threshold, best.default_left)) {
          if (nl < best.left.count) lrows[nl] = row;
          ++nl;
        } else {
          if (nr < best.right.count) rrows[nr] = row;
          ++nr;
        }
      }
      if (nl != best.left.count || nr != best.right.count) {
        free(lrows); free(rrows);
        rc = fail(ORC_TRAINING_ERROR, "Sample partition counts do not match histogram statistics");
        break;
      }
      /* ApplySplit, tree_structure.cpp:118-148 */
      double lv = 0.0, rv = 0.0;
      uint32_t li, ri;
      rc = bounded_leaf(p, &best.left, best.ll, best.lu, &lv);
      if (rc == ORC_OK) rc = append_node(tree, leaf_node(lv), &li);
      if (rc == ORC_OK) rc = bounded_leaf(p, &best.right, best.rl, best.ru, &rv);
      if (rc == ORC_OK) rc = append_node(tree, leaf_node(rv), &ri);
      if (rc != ORC_OK) { free(lrows); free(rrows); break; }
      orc_tree_node* parent = &tree->nodes[a->node_index];
      parent->feature_index = best.feature;
      parent->threshold_bin = best.threshold;
      parent->left_child = li;
      parent->right_child = ri;
      parent->leaf_value = 0.0;
      parent->gain = best.gain;
      parent->default_left = (uint8_t)best.default_left;
      parent->flags = 0;
      ++leaf_count;
      /* Children, tree.cpp:96-117 (ExtendInteractionPath, tree_interactions.cpp:47-55) */
      const uint32_t child_depth = a->depth + 1;
      uint32_t* path = (uint32_t*)malloc((a->n_path + 1) * sizeof(uint32_t));
      memcpy(path, a->path, a->n_path * sizeof(uint32_t));
      uint32_t n_path = a->n_path;
      int seen = 0;
      for (uint32_t k = 0; k < n_path; ++k) seen |= path[k] == best.feature;
      if (!seen) path[n_path++] = best.feature;
      active_t* L = &next[n_next++];
      active_t* R = &next[n_next++];
      L->node_index = li; L->depth = child_depth; L->rows = lrows; L->n_rows = nl;
      L->stats = best.left; L->lo = best.ll; L->hi = best.lu;
      L->path = path; L->n_path = n_path;
      R->node_index = ri; R->depth = child_depth; R->rows = rrows; R->n_rows = nr;
      R->stats = best.right; R->lo = best.rl; R->hi = best.ru;
      R->path = (uint32_t*)malloc((n_path ? n_path : 1) * sizeof(uint32_t));
      memcpy(R->path, path, n_path * sizeof(uint32_t));
      R->n_path = n_path;
      if (child_depth < p->max_depth) {
        /* Smaller child built, sibling by subtraction (tree.cpp:109-143). */
        const int build_left = best.left.count <= best.right.count;
        active_t* built = build_left ? L : R;
        active_t* other = build_left ? R : L;
        rc = build_hist(x, built->rows, built->n_rows, &built->hist);
        if (rc == ORC_OK) rc = subtract_hist(x, &a->hist, &built->hist, &other->hist);
      }
    }
    for (uint64_t i = 0; i < n_cur; ++i) free_active(&cur[i]);
    free(cur);
    cur = next;
    n_cur = n_next;
  }
  for (uint64_t i = 0; i < n_cur; ++i) free_active(&cur[i]);
  free(cur);
  free(miss);
  return rc;
}

static int make_ctx(const dataset_t* d, const orc_params* p, ctx_t* x) {
  memset(x, 0, sizeof *x);
  x->d = d;
  x->p = p;
  x->offset = (uint64_t*)malloc(d->features * sizeof(uint64_t));
  uint64_t t = 0;
  for (uint32_t f = 0; f < d->features; ++f) { x->offset[f] = t; t += d->bin_count[f]; }
  x->n_bins = t;
  return ORC_OK;
}

/* TrainLeafWiseRegressionTree, tree_leafwise.cpp:56-142: repeatedly split the active
   leaf with the largest gain (the smaller node index on equal gains) until max_leaves;
   leaves at max_depth stay active but never split. A leaf's best split depends only on
   its own rows, so it is found once and kept until the leaf is split. */
static int grow_leaf_wise(const ctx_t* x, tree_t* tree) {
  const dataset_t* d = x->d;
  const orc_params* p = x->p;
  int rc = ORC_OK;
  const uint32_t max_leaves = effective_max_leaves(p);
  const uint32_t max_active = p->max_active_leaves ? p->max_active_leaves : max_leaves;
  uint64_t cap = 16, n_act = 1;
  active_t* act = (active_t*)calloc(cap, sizeof(active_t));
  candidate_t* cand = (candidate_t*)calloc(cap, sizeof(candidate_t));
  int* scored = (int*)calloc(cap, sizeof(int));
  act[0].rows = (uint64_t*)malloc(d->rows * sizeof(uint64_t));
  for (uint64_t r = 0; r < d->rows; ++r) act[0].rows[r] = r;
  act[0].n_rows = d->rows;
  act[0].lo = -INFINITY;
  act[0].hi = INFINITY;
  rc = sum_rows(x, act[0].rows, d->rows, &act[0].stats);
  if (rc == ORC_OK) {
    double leaf;
    rc = bounded_leaf(p, &act[0].stats, -INFINITY, INFINITY, &leaf);
    uint32_t idx;
    if (rc == ORC_OK) rc = append_node(tree, leaf_node(leaf), &idx);
  }
  uint32_t leaf_count = 1;
  stats_t* miss = (stats_t*)malloc(d->features * sizeof(stats_t));
  while (rc == ORC_OK && n_act > 0 && leaf_count < max_leaves) {
    if (n_act > max_active) { rc = fail(ORC_TRAINING_ERROR, "active leaf queue exceeded max_active_leaves"); break; }
    int64_t best = -1;
    for (uint64_t i = 0; i < n_act && rc == ORC_OK; ++i) {
      active_t* a = &act[i];
      if (a->depth >= p->max_depth) continue;
      if (a->hist.fp == NULL && a->hist.fx == NULL) rc = build_hist(x, a->rows, a->n_rows, &a->hist);
      if (rc != ORC_OK) break;
      if (!scored[i]) {  /* PrepareSplitRows, tree_split.cpp:236-291 */
        node_missing(x, a, &a->hist, miss);
        rc = find_best_split(x, a, &a->hist, miss, &cand[i]);
        scored[i] = 1;
        if (rc != ORC_OK) break;
      }
      if (!cand[i].valid) continue;
      /* IsBetterLeafWiseCandidate, tree_leafwise.cpp:16-27 */
      if (best < 0 || cand[i].gain > cand[best].gain ||
          (cand[i].gain == cand[best].gain && a->node_index < act[best].node_index)) {
        /* The superseded best leaf's histogram was moved into the step's best slot and is
           overwritten there (tree_leafwise.cpp:94-100): that leaf is rebuilt from its rows
           the next time it is evaluated, and its split found again. */
        if (best >= 0) {
          free_hist(&act[best].hist);
          memset(&act[best].hist, 0, sizeof act[best].hist);
          scored[best] = 0;
        }
        best = (int64_t)i;
      }
    }
    if (rc != ORC_OK || best < 0) break;
    active_t chosen = act[best];
    const candidate_t split = cand[best];
    for (uint64_t i = (uint64_t)best; i + 1 < n_act; ++i) {  /* erase, order kept */
      act[i] = act[i + 1];
      cand[i] = cand[i + 1];
      scored[i] = scored[i + 1];
    }
    --n_act;
    uint64_t* lrows = (uint64_t*)malloc((split.left.count ? split.left.count : 1) * sizeof(uint64_t));
    uint64_t* rrows = (uint64_t*)malloc((split.right.count ? split.right.count : 1) * sizeof(uint64_t));
    uint64_t nl = 0, nr = 0;
    for (uint64_t k = 0; k < chosen.n_rows; ++k) {
      const uint64_t row = chosen.rows[k];
      if (goes_left(d, row, split.feature, split.threshold, split.default_left)) {
        if (nl < split.left.count) lrows[nl] = row;
        ++nl;
      } else {
        if (nr < split.right.count) rrows[nr] = row;
        ++nr;
      }
    }
    if (nl != split.left.count || nr != split.right.count) {
      free(lrows); free(rrows); free_active(&chosen);
      rc = fail(ORC_TRAINING_ERROR, "Sample partition counts do not match histogram statistics");
      break;
    }
    double lv = 0.0, rv = 0.0;  /* ApplySplit, tree_structure.cpp:118-148 */
    uint32_t li = 0, ri = 0;
    rc = bounded_leaf(p, &split.left, split.ll, split.lu, &lv);
    if (rc == ORC_OK) rc = append_node(tree, leaf_node(lv), &li);
    if (rc == ORC_OK) rc = bounded_leaf(p, &split.right, split.rl, split.ru, &rv);
    if (rc == ORC_OK) rc = append_node(tree, leaf_node(rv), &ri);
    if (rc != ORC_OK) { free(lrows); free(rrows); free_active(&chosen); break; }
    orc_tree_node* parent = &tree->nodes[chosen.node_index];
    parent->feature_index = split.feature;
    parent->threshold_bin = split.threshold;
    parent->left_child = li;
    parent->right_child = ri;
    parent->leaf_value = 0.0;
    parent->gain = split.gain;
    parent->default_left = (uint8_t)split.default_left;
    parent->flags = 0;
    ++leaf_count;
    const uint32_t child_depth = chosen.depth + 1;
    uint32_t* path = (uint32_t*)malloc((chosen.n_path + 1) * sizeof(uint32_t));
    memcpy(path, chosen.path, chosen.n_path * sizeof(uint32_t));
    uint32_t n_path = chosen.n_path;
    int seen = 0;
    for (uint32_t k = 0; k < n_path; ++k) seen |= path[k] == split.feature;
    if (!seen) path[n_path++] = split.feature;
    active_t L, R;
    memset(&L, 0, sizeof L);
    memset(&R, 0, sizeof R);
    L.node_index = li; L.depth = child_depth; L.rows = lrows; L.n_rows = nl;
    L.stats = split.left; L.lo = split.ll; L.hi = split.lu; L.path = path; L.n_path = n_path;
    R.node_index = ri; R.depth = child_depth; R.rows = rrows; R.n_rows = nr;
    R.stats = split.right; R.lo = split.rl; R.hi = split.ru;
    R.path = (uint32_t*)malloc((n_path ? n_path : 1) * sizeof(uint32_t));
    memcpy(R.path, path, n_path * sizeof(uint32_t));
    R.n_path = n_path;
    if (child_depth < p->max_depth) {  /* CacheChildHistograms, tree_leafwise.cpp:29-52 */
      const int build_left = split.left.count <= split.right.count;
      active_t* built = build_left ? &L : &R;
      active_t* other = build_left ? &R : &L;
      rc = build_hist(x, built->rows, built->n_rows, &built->hist);
      if (rc == ORC_OK) rc = subtract_hist(x, &chosen.hist, &built->hist, &other->hist);
    }
    free_active(&chosen);
    if (rc != ORC_OK) { free_active(&L); free_active(&R); break; }
    if (!(n_act + 2 <= max_active || leaf_count >= max_leaves)) {
      free_active(&L); free_active(&R);
      rc = fail(ORC_TRAINING_ERROR, "leaf-wise active queue reached max_active_leaves");
      break;
    }
    if (n_act + 2 > cap) {
      cap *= 2;
      act = (active_t*)realloc(act, cap * sizeof(active_t));
      cand = (candidate_t*)realloc(cand, cap * sizeof(candidate_t));
      scored = (int*)realloc(scored, cap * sizeof(int));
    }
    act[n_act] = L;
    scored[n_act++] = 0;
    act[n_act] = R;
    scored[n_act++] = 0;
  }
  for (uint64_t i = 0; i < n_act; ++i) free_active(&act[i]);
  free(act); free(cand); free(scored); free(miss);
  return rc;
}

/* TrainSingleRegressionTree, tree.cpp:151-177. */
static int train_tree(ctx_t* x, tree_t** out) {
  const orc_params* p = x->p;
  TRY(validate_tree_params(p));
  if (p->n_monotonic != 0 && p->n_monotonic != x->d->features)
    return fail(ORC_TRAINING_ERROR, "monotonic_constraints length must match feature count");
  for (uint32_t i = 0; i < p->n_monotonic; ++i)
    if (p->monotonic_constraints[i] < -1 || p->monotonic_constraints[i] > 1)
      return fail(ORC_TRAINING_ERROR, "monotonic_constraints values must be -1, 0, or 1");
  for (uint32_t g = 0; g < p->n_interaction_groups; ++g) { /* tree_interactions.cpp:57-70 */
    if (p->interaction_offsets[g + 1] == p->interaction_offsets[g])
      return fail(ORC_TRAINING_ERROR, "interaction constraint groups must be non-empty");
    for (uint32_t i = p->interaction_offsets[g]; i < p->interaction_offsets[g + 1]; ++i)
      if (p->interaction_features[i] >= x->d->features)
        return fail(ORC_TRAINING_ERROR, "interaction constraint feature index out of range");
  }
  if (p->growth_strategy > 1) return fail(ORC_TRAINING_ERROR, "unknown growth strategy");
  tree_t* t = (tree_t*)calloc(1, sizeof(tree_t));
  t->features = x->d->features;
  const int rc = p->growth_strategy == 1 ? grow_leaf_wise(x, t) : grow_level_wise(x, t);
  if (rc != ORC_OK) { free(t->nodes); free(t); return rc; }
  *out = t;
  return ORC_OK;
}

int orc_train_single_tree(const void* dataset, const double* pairs, uint64_t n,
                          const orc_params* p, void** out) {
  const dataset_t* d = (const dataset_t*)dataset;
  if (d->rows != n)
    return fail(ORC_TRAINING_ERROR, "Gradient count does not match binned dataset row count");
  ctx_t x;
  make_ctx(d, p, &x);
  x.pairs = pairs;
  tree_t* t = NULL;
  const int rc = train_tree(&x, &t);
  free(x.offset);
  *out = t;
  return rc;
}

int orc_train_single_tree_fixed(const void* dataset, const float* pairs32, uint64_t n,
                                int32_t kg, int32_t kh, const orc_params* p, void** out) {
  const dataset_t* d = (const dataset_t*)dataset;
  if (d->rows != n)
    return fail(ORC_TRAINING_ERROR, "Gradient count does not match binned dataset row count");
  ctx_t x;
  make_ctx(d, p, &x);
  x.pairs32 = pairs32;
  x.kg = kg;
  x.kh = kh;
  x.mode.fixed = 1;
  x.mode.inv_g = ldexp(1.0, -kg);
  x.mode.inv_h = ldexp(1.0, -kh);
  tree_t* t = NULL;
  const int rc = train_tree(&x, &t);
  free(x.offset);
  *out = t;
  return rc;
}

uint32_t orc_tree_node_count(const void* tree) { return ((const tree_t*)tree)->n; }

int orc_tree_nodes(const void* tree, orc_tree_node* out) {
  const tree_t* t = (const tree_t*)tree;
  memcpy(out, t->nodes, t->n * sizeof(orc_tree_node));
  return ORC_OK;
}

/* RegressionTree::Predict, tree.cpp:179-214. */
static int tree_predict(const tree_t* t, const dataset_t* d, double* out) {
  if (t->n == 0) return fail(ORC_TRAINING_ERROR, "Tree model has no root node");
  if (d->features != t->features)
    return fail(ORC_TRAINING_ERROR, "Prediction feature count does not match the tree model");
  for (uint64_t row = 0; row < d->rows; ++row) {
    uint32_t node = 0;
    uint64_t visited = 0;
    for (;;) {
      if (node >= t->n || ++visited > t->n)
        return fail(ORC_TRAINING_ERROR, "Tree node index is out of bounds or the structure contains a cycle");
      const orc_tree_node* nd = &t->nodes[node];
      if (nd->flags & 1u) {
        if (!isfinite(nd->leaf_value)) return fail(ORC_TRAINING_ERROR, "Tree leaf value is not finite");
        out[row] = nd->leaf_value;
        break;
      }
      if (nd->feature_index >= t->features)
        return fail(ORC_TRAINING_ERROR, "Tree branch feature index is out of bounds");
      node = goes_left(d, row, nd->feature_index, nd->threshold_bin, nd->default_left)
                 ? nd->left_child : nd->right_child;
    }
  }
  return ORC_OK;
}

int orc_tree_predict(const void* tree, const void* dataset, double* out) {
  return tree_predict((const tree_t*)tree, (const dataset_t*)dataset, out);
}

void orc_tree_free(void* tree) {
  tree_t* t = (tree_t*)tree;
  if (t) { free(t->nodes); free(t); }
}

/* ------------------------------------------------------------------------------------
 * Boosting (trainer.cpp:22-42, 226-282)
 * ---------------------------------------------------------------------------------- */
typedef struct {
  double base_score, learning_rate;
  uint32_t n_trees;
  tree_t** trees;
  uint32_t features, max_bins;
  float* boundaries;
  uint64_t n_boundaries;
} model_t;

void orc_model_free(void* m) {
  model_t* model = (model_t*)m;
  if (!model) return;
  for (uint32_t i = 0; i < model->n_trees; ++i) orc_tree_free(model->trees[i]);
  free(model->trees);
  free(model->boundaries);
  free(model);
}

static int validate_training_params(const orc_params* p) { /* trainer.cpp:22-42 */
  if (p->n_estimators == 0) return fail(ORC_TRAINING_ERROR, "n_estimators must be at least 1");
  if (!isfinite(p->learning_rate) || p->learning_rate <= 0.0 || p->learning_rate > 1.0)
    return fail(ORC_TRAINING_ERROR, "learning_rate must be in (0, 1]");
  if (p->max_bins < 2 || p->max_bins > 65536)
    return fail(ORC_TRAINING_ERROR, "max_bins must be in [2, 65536]");
  if (!isfinite(p->objective_alpha) || p->objective_alpha <= 0.0 || p->objective_alpha >= 1.0)
    return fail(ORC_TRAINING_ERROR, "quantile alpha must be in (0, 1)");
  if (!isfinite(p->tweedie_variance_power) || p->tweedie_variance_power <= 1.0 ||
      p->tweedie_variance_power >= 2.0)
    return fail(ORC_TRAINING_ERROR, "tweedie variance power must be in (1, 2)");
  return ORC_OK;
}

int orc_train_regressor_mode(const void* dataset, const double* labels, const double* weights,
                             uint64_t n, const orc_params* p, int hist_mode, void** out) {
  const dataset_t* d = (const dataset_t*)dataset;
  TRY(validate_training_params(p));
  if (d->rows != n || d->max_bins != p->max_bins)
    return fail(ORC_TRAINING_ERROR, "Training data, labels, or max_bins contract does not match");
  double total;
  TRY(validate_weights(weights, n, &total));
  model_t* m = (model_t*)calloc(1, sizeof(model_t));
  int rc = base_score(p, labels, weights, n, &m->base_score);
  m->learning_rate = p->learning_rate;
  m->features = d->features;
  m->max_bins = d->max_bins;
  m->n_boundaries = d->n_boundaries;
  m->boundaries = (float*)malloc((d->n_boundaries ? d->n_boundaries : 1) * sizeof(float));
  memcpy(m->boundaries, d->boundaries, d->n_boundaries * sizeof(float));
  m->trees = (tree_t**)calloc(p->n_estimators, sizeof(tree_t*));
  double* preds = (double*)malloc(n * sizeof(double));
  double* pairs = (double*)malloc(2 * n * sizeof(double));
  float* pairs32 = (float*)malloc(2 * n * sizeof(float));
  double* update = (double*)malloc(n * sizeof(double));
  for (uint64_t i = 0; i < n; ++i) preds[i] = m->base_score;
  ctx_t x;
  make_ctx(d, p, &x);
  for (uint32_t round = 0; round < p->n_estimators && rc == ORC_OK; ++round) {
    rc = orc_gradients(p->objective, p->objective_alpha, p->tweedie_variance_power, labels,
                       preds, n, pairs);
    if (rc == ORC_OK) rc = apply_sample_weights(pairs, weights, n);
    if (rc != ORC_OK) break;
    x.pairs = pairs;
    if (hist_mode == ORC_HIST_FIXED) {
      for (uint64_t i = 0; i < 2 * n; ++i) pairs32[i] = (float)pairs[i];
      rc = orc_fixed_scales(pairs32, n, &x.kg, &x.kh);
      if (rc != ORC_OK) break;
      x.pairs32 = pairs32;
      x.mode.fixed = 1;
      x.mode.inv_g = ldexp(1.0, -x.kg);
      x.mode.inv_h = ldexp(1.0, -x.kh);
    }
    tree_t* t = NULL;
    rc = train_tree(&x, &t);
    if (rc != ORC_OK) break;
    m->trees[m->n_trees++] = t;
    rc = tree_predict(t, d, update);
    for (uint64_t i = 0; i < n && rc == ORC_OK; ++i) {
      preds[i] += p->learning_rate * update[i];
      if (!isfinite(preds[i])) rc = fail(ORC_TRAINING_ERROR, "Boosting prediction update overflowed");
    }
  }
  free(x.offset);
  free(preds); free(pairs); free(pairs32); free(update);
  if (rc != ORC_OK) { orc_model_free(m); return rc; }
  *out = m;
  return ORC_OK;
}

int orc_train_regressor(const void* dataset, const double* labels, const double* weights,
                        uint64_t n, const orc_params* p, void** out) {
  return orc_train_regressor_mode(dataset, labels, weights, n, p, ORC_HIST_FP64, out);
}

uint32_t orc_model_tree_count(const void* m) { return ((const model_t*)m)->n_trees; }
double orc_model_base_score(const void* m) { return ((const model_t*)m)->base_score; }
uint32_t orc_model_tree_node_count(const void* m, uint32_t t) {
  return ((const model_t*)m)->trees[t]->n;
}
int orc_model_tree_nodes(const void* m, uint32_t t, orc_tree_node* out) {
  const model_t* model = (const model_t*)m;
  if (t >= model->n_trees) return fail(ORC_OTHER_ERROR, "tree index out of range");
  return orc_tree_nodes(model->trees[t], out);
}

/* RegressionModel::Predict, trainer.cpp:268-282. */
int orc_model_predict(const void* m, const void* dataset, double* out) {
  const model_t* model = (const model_t*)m;
  const dataset_t* d = (const dataset_t*)dataset;
  if (d->features != model->features || d->max_bins != model->max_bins ||
      d->n_boundaries != model->n_boundaries ||
      memcmp(d->boundaries, model->boundaries, d->n_boundaries * sizeof(float)) != 0)
    return fail(ORC_TRAINING_ERROR, "Prediction data does not use the model's frozen binned schema");
  double* update = (double*)malloc(d->rows * sizeof(double));
  for (uint64_t i = 0; i < d->rows; ++i) out[i] = model->base_score;
  for (uint32_t t = 0; t < model->n_trees; ++t) {
    const int rc = tree_predict(model->trees[t], d, update);
    if (rc != ORC_OK) { free(update); return rc; }
    for (uint64_t i = 0; i < d->rows; ++i) out[i] += model->learning_rate * update[i];
  }
  free(update);
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------
 * Native softmax boosting (multiclass_trainer.cpp:104-149): per round, one tree per class
 * in class order, each fitted to the softmax gradients of the current margins, which
 * include the earlier classes' trees of the same round.
 * ---------------------------------------------------------------------------------- */
typedef struct {
  uint32_t class_count;
  double learning_rate;
  double* base_scores;
  uint32_t n_trees;
  tree_t** trees;
  uint32_t features, max_bins;
  float* boundaries;
  uint64_t n_boundaries;
} softmax_t;

void orc_softmax_free(void* m) {
  softmax_t* model = (softmax_t*)m;
  if (!model) return;
  for (uint32_t i = 0; i < model->n_trees; ++i) orc_tree_free(model->trees[i]);
  free(model->trees);
  free(model->base_scores);
  free(model->boundaries);
  free(model);
}

/* ComputeMulticlassSoftmaxGradients + SoftmaxProbabilities (objective.cpp:130-152,
   242-287): pairs for target_class from margins [rows][class_count]. */
static int softmax_gradients(const double* labels, const double* margins, uint64_t n,
                             uint32_t K, uint32_t target, double* probs, double* out) {
  for (uint64_t r = 0; r < n; ++r) {
    const double label = labels[r];
    if (!isfinite(label)) return fail(ORC_TRAINING_ERROR, "softmax label must be finite");
    if (floor(label) != label || label < 0.0 || label >= (double)K)
      return fail(ORC_TRAINING_ERROR, "softmax labels must be encoded class ids");
    double maximum = -INFINITY;
    for (uint32_t k = 0; k < K; ++k) {
      const double m = margins[r * K + k];
      if (!isfinite(m)) return fail(ORC_TRAINING_ERROR, "softmax margin must be finite");
      if (m > maximum) maximum = m;
    }
    double normalizer = 0.0;
    for (uint32_t k = 0; k < K; ++k) {
      probs[k] = exp(margins[r * K + k] - maximum);
      normalizer += probs[k];
    }
    if (!isfinite(normalizer) || normalizer <= 0.0)
      return fail(ORC_TRAINING_ERROR, "softmax normalizer must be finite and positive");
    const double p = probs[target] / normalizer;
    const double indicator = (uint32_t)label == target ? 1.0 : 0.0;
    const double g = p - indicator, h = p * (1.0 - p);
    if (!isfinite(g) || !isfinite(h) || h < 0.0)
      return fail(ORC_TRAINING_ERROR, "softmax gradient/Hessian overflowed");
    out[2 * r] = g;
    out[2 * r + 1] = h;
  }
  return ORC_OK;
}

int orc_train_softmax_mode(const void* dataset, const double* labels, const double* weights,
                           uint64_t n, const orc_params* p, uint32_t K, int hist_mode,
                           void** out) {
  const dataset_t* d = (const dataset_t*)dataset;
  TRY(validate_training_params(p));
  if (d->rows != n || d->max_bins != p->max_bins)
    return fail(ORC_TRAINING_ERROR, "training data, labels, or max_bins contract mismatch");
  double total;
  TRY(validate_weights(weights, n, &total));
  if (K < 2) return fail(ORC_TRAINING_ERROR, "softmax class_count must be at least two");
  for (uint64_t r = 0; r < n; ++r) {  /* ValidateMulticlassLabels, multiclass_trainer.cpp:22-37 */
    if (!isfinite(labels[r])) return fail(ORC_TRAINING_ERROR, "softmax labels must be finite");
    if (floor(labels[r]) != labels[r] || labels[r] < 0.0 || labels[r] >= (double)K)
      return fail(ORC_TRAINING_ERROR, "softmax labels must be encoded class ids");
  }
  softmax_t* m = (softmax_t*)calloc(1, sizeof(softmax_t));
  m->class_count = K;
  m->learning_rate = p->learning_rate;
  m->features = d->features;
  m->max_bins = d->max_bins;
  m->n_boundaries = d->n_boundaries;
  m->boundaries = (float*)malloc((d->n_boundaries ? d->n_boundaries : 1) * sizeof(float));
  memcpy(m->boundaries, d->boundaries, d->n_boundaries * sizeof(float));
  m->base_scores = (double*)calloc(K, sizeof(double));
  m->trees = (tree_t**)calloc((size_t)p->n_estimators * K, sizeof(tree_t*));
  int rc = ORC_OK;
  /* WeightedClassBaseScores, multiclass_trainer.cpp:39-67. */
  double* cw = (double*)calloc(K, sizeof(double));
  for (uint64_t r = 0; r < n && rc == ORC_OK; ++r) {
    const uint32_t c = (uint32_t)labels[r];
    cw[c] += weights[r];
    if (!isfinite(cw[c])) rc = fail(ORC_TRAINING_ERROR, "softmax class prior overflowed");
  }
  for (uint32_t k = 0; k < K && rc == ORC_OK; ++k) {
    double prob = cw[k] / total;
    if (prob < 1e-15) prob = 1e-15;
    m->base_scores[k] = log(prob);
    if (!isfinite(m->base_scores[k])) rc = fail(ORC_TRAINING_ERROR, "softmax base score is not finite");
  }
  free(cw);
  double* margins = (double*)malloc(n * K * sizeof(double));
  double* pairs = (double*)malloc(2 * n * sizeof(double));
  float* pairs32 = (float*)malloc(2 * n * sizeof(float));
  double* update = (double*)malloc(n * sizeof(double));
  double* probs = (double*)malloc(K * sizeof(double));
  for (uint64_t r = 0; r < n; ++r)
    for (uint32_t k = 0; k < K; ++k) margins[r * K + k] = m->base_scores[k];
  ctx_t x;
  make_ctx(d, p, &x);
  for (uint32_t round = 0; round < p->n_estimators && rc == ORC_OK; ++round) {
    for (uint32_t k = 0; k < K && rc == ORC_OK; ++k) {
      rc = softmax_gradients(labels, margins, n, K, k, probs, pairs);
      if (rc == ORC_OK) rc = apply_sample_weights(pairs, weights, n);
      if (rc != ORC_OK) break;
      x.pairs = pairs;
      x.mode.fixed = 0;
      if (hist_mode == ORC_HIST_FIXED) {
        for (uint64_t i = 0; i < 2 * n; ++i) pairs32[i] = (float)pairs[i];
        rc = orc_fixed_scales(pairs32, n, &x.kg, &x.kh);
        if (rc != ORC_OK) break;
        x.pairs32 = pairs32;
        x.mode.fixed = 1;
        x.mode.inv_g = ldexp(1.0, -x.kg);
        x.mode.inv_h = ldexp(1.0, -x.kh);
      }
      tree_t* t = NULL;
      rc = train_tree(&x, &t);
      if (rc != ORC_OK) break;
      m->trees[m->n_trees++] = t;
      rc = tree_predict(t, d, update);
      for (uint64_t r = 0; r < n && rc == ORC_OK; ++r) {  /* AddClassUpdate */
        double* margin = &margins[r * K + k];
        *margin += p->learning_rate * update[r];
        if (!isfinite(*margin)) rc = fail(ORC_TRAINING_ERROR, "softmax margin update overflowed");
      }
    }
  }
  free(x.offset);
  free(margins); free(pairs); free(pairs32); free(update); free(probs);
  if (rc != ORC_OK) { orc_softmax_free(m); return rc; }
  *out = m;
  return ORC_OK;
}

int orc_train_softmax(const void* dataset, const double* labels, const double* weights,
                      uint64_t n, const orc_params* p, uint32_t K, void** out) {
  return orc_train_softmax_mode(dataset, labels, weights, n, p, K, ORC_HIST_FP64, out);
}

uint32_t orc_softmax_tree_count(const void* m) { return ((const softmax_t*)m)->n_trees; }
uint32_t orc_softmax_class_count(const void* m) { return ((const softmax_t*)m)->class_count; }
int orc_softmax_base_scores(const void* m, double* out) {
  const softmax_t* s = (const softmax_t*)m;
  memcpy(out, s->base_scores, s->class_count * sizeof(double));
  return ORC_OK;
}
uint32_t orc_softmax_tree_node_count(const void* m, uint32_t t) {
  return ((const softmax_t*)m)->trees[t]->n;
}
int orc_softmax_tree_nodes(const void* m, uint32_t t, orc_tree_node* out) {
  const softmax_t* s = (const softmax_t*)m;
  if (t >= s->n_trees) return fail(ORC_OTHER_ERROR, "tree index out of range");
  return orc_tree_nodes(s->trees[t], out);
}

/* MulticlassModel::PredictMargins, multiclass_trainer.cpp:212-235: [rows][class_count]. */
int orc_softmax_predict_margins(const void* m, const void* dataset, double* out) {
  const softmax_t* s = (const softmax_t*)m;
  const dataset_t* d = (const dataset_t*)dataset;
  if (d->features != s->features || d->max_bins != s->max_bins ||
      d->n_boundaries != s->n_boundaries ||
      memcmp(d->boundaries, s->boundaries, d->n_boundaries * sizeof(float)) != 0)
    return fail(ORC_TRAINING_ERROR, "prediction data does not use the frozen model binning schema");
  const uint32_t K = s->class_count;
  for (uint64_t r = 0; r < d->rows; ++r)
    for (uint32_t k = 0; k < K; ++k) out[r * K + k] = s->base_scores[k];
  double* update = (double*)malloc(d->rows * sizeof(double));
  for (uint32_t t = 0; t < s->n_trees; ++t) {
    const int rc = tree_predict(s->trees[t], d, update);
    if (rc != ORC_OK) { free(update); return rc; }
    const uint32_t k = t % K;
    for (uint64_t r = 0; r < d->rows; ++r) {
      out[r * K + k] += s->learning_rate * update[r];
      if (!isfinite(out[r * K + k])) { free(update); return fail(ORC_TRAINING_ERROR, "softmax margin update overflowed"); }
    }
  }
  free(update);
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------
 * Finer-grained hooks mirroring MpsBackend::ScanSplitsForTest / PartitionRowsForTest
 * (mps_split_partition.mm:14-236) with full reference semantics.
 * ---------------------------------------------------------------------------------- */
int orc_scan_splits(const void* dataset, const double* pairs, uint64_t n, const uint64_t* rows,
                    uint64_t n_rows, const orc_params* p, orc_split_candidate* out) {
  const dataset_t* d = (const dataset_t*)dataset;
  if (d->rows != n)
    return fail(ORC_TRAINING_ERROR, "Gradient count does not match binned dataset row count");
  TRY(validate_tree_params(p));
  ctx_t x;
  make_ctx(d, p, &x);
  x.pairs = pairs;
  active_t a;
  memset(&a, 0, sizeof a);
  a.rows = (uint64_t*)rows;
  a.n_rows = n_rows;
  a.lo = -INFINITY;
  a.hi = INFINITY;
  node_hist_t h;
  stats_t* miss = (stats_t*)malloc(d->features * sizeof(stats_t));
  int rc = sum_rows(&x, rows, n_rows, &a.stats);
  if (rc == ORC_OK) rc = build_hist(&x, rows, n_rows, &h);
  if (rc == ORC_OK) node_missing(&x, &a, &h, miss);
  for (uint32_t f = 0; f < d->features && rc == ORC_OK; ++f) {
    candidate_t best;
    memset(&best, 0, sizeof best);
    rc = scan_feature(&x, &h, miss, &a.stats, a.lo, a.hi, 0, 0, f, &best);
    orc_split_candidate* o = &out[f];
    memset(o, 0, sizeof *o);
    o->valid = (uint32_t)best.valid;
    o->feature = f;
    if (best.valid) {
      o->threshold_bin = best.threshold;
      o->default_left = (uint32_t)best.default_left;
      o->left_count = best.left.count;
      o->right_count = best.right.count;
      o->left_gradient_sum = best.left.g;
      o->left_hessian_sum = best.left.h;
      o->right_gradient_sum = best.right.g;
      o->right_hessian_sum = best.right.h;
      o->gain = best.gain;
    }
  }
  free_hist(&h);
  free(miss);
  free(x.offset);
  return rc;
}

int orc_partition_rows(const void* dataset, const uint64_t* rows, uint64_t n_rows,
                       uint32_t feature, uint32_t threshold_bin, int default_left,
                       uint64_t* left_out, uint64_t* right_out, uint64_t* n_left) {
  const dataset_t* d = (const dataset_t*)dataset;
  if (n_rows == 0) return fail(ORC_TRAINING_ERROR, "Partition row set must not be empty");
  if (feature >= d->features || threshold_bin >= d->bin_count[feature])
    return fail(ORC_TRAINING_ERROR, "Partition feature or threshold is out of bounds");
  uint64_t nl = 0, nr = 0;
  for (uint64_t i = 0; i < n_rows; ++i) {
    if (rows[i] >= d->rows) return fail(ORC_TRAINING_ERROR, "partition row index is out of bounds");
    if (goes_left(d, rows[i], feature, threshold_bin, default_left)) left_out[nl++] = rows[i];
    else right_out[nr++] = rows[i];
  }
  *n_left = nl;
  return ORC_OK;
}
