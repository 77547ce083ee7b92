// Host quantile binning with the reference's semantics, parallel over features.
//
// Semantics follow src/core/binned_dataset.cpp:
//   * NaN is missing: excluded from quantiles, stored as bin 0 plus a missing flag
//     (126-188); Inf is an error (50-81); float64 input must fit in float32.
//   * Boundaries: sort the non-missing values, take the value at rank
//     ceil(part * m / desired) - 1 for part = 1..desired-1 with desired = min(max_bins, m),
//     keep it when it is below the maximum and above the previous boundary (83-118).
//   * bin = lower_bound(boundaries, value): a value equal to a boundary stays in the
//     lower bin (166-176); storage is u8 when max_bins <= 256, else u16.
// The work for each feature is independent, so features are spread over host threads.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "host_errors.h"

namespace mpsb {
namespace {

struct View {
  const uint8_t* data;
  int scalar_type;
  uint64_t rows;
  uint32_t features;
  uint64_t rs, cs;
};

float read_value(const View& v, uint64_t row, uint32_t feature) {
  const uint8_t* p = v.data + row * v.rs + uint64_t(feature) * v.cs;
  if (v.scalar_type == 1) {
    float x;
    std::memcpy(&x, p, sizeof x);
    if (std::isnan(x)) return x;
    if (!std::isfinite(x)) throw DataError("Input matrix contains Inf");
    return x;
  }
  double x;
  std::memcpy(&x, p, sizeof x);
  if (std::isnan(x)) return std::numeric_limits<float>::quiet_NaN();
  if (!std::isfinite(x)) throw DataError("Input matrix contains Inf");
  constexpr double kMax = double(std::numeric_limits<float>::max());
  if (x > kMax || x < -kMax) throw DataError("float64 input value exceeds the finite float32 range");
  return float(x);
}

uint64_t quantile_rank(uint64_t part, uint64_t total, uint64_t divisor) {
  const uint64_t whole = part * (total / divisor);
  const uint64_t numerator = part * (total % divisor);
  return whole + numerator / divisor + (numerator % divisor != 0 ? 1 : 0) - 1;
}

void validate(const View& v, uint32_t max_bins) {
  if (v.data == nullptr) throw DataError("Input matrix data must not be null");
  if (v.rows == 0 || v.features == 0)
    throw DataError("Input matrix must contain at least one row and one feature");
  if (max_bins < 2 || max_bins > 65536) throw DataError("max_bins must be in [2, 65536]");
  if (v.scalar_type != 1 && v.scalar_type != 2) throw DataError("Input scalar type is not supported");
  const uint64_t item = v.scalar_type == 2 ? 8 : 4;
  if (v.rs < item || v.cs < item) throw DataError("Input matrix stride is smaller than the element size");
  uint64_t a, b, c;
  if (__builtin_mul_overflow(v.rows - 1, v.rs, &a) ||
      __builtin_mul_overflow(uint64_t(v.features - 1), v.cs, &b) ||
      __builtin_add_overflow(a, b, &c) || __builtin_add_overflow(c, item, &c) ||
      __builtin_mul_overflow(v.rows, uint64_t(v.features), &a))
    throw DataError("input matrix maximum offset: multiplication overflow");
}

template <typename F>
void parallel_features(uint32_t features, uint32_t n_threads, F&& body) {
  uint32_t workers = n_threads ? n_threads : std::max(1u, std::thread::hardware_concurrency());
  workers = std::min(workers, features);
  std::atomic<uint32_t> next{0};
  std::vector<std::string> errors(workers);
  std::vector<int> codes(workers, 0);
  auto run = [&](uint32_t w) {
    try {
      for (uint32_t f = next.fetch_add(1); f < features; f = next.fetch_add(1)) body(f);
    } catch (const Error& e) {
      codes[w] = e.code;
      errors[w] = e.what();
    } catch (const std::exception& e) {
      codes[w] = 4;
      errors[w] = e.what();
    }
  };
  std::vector<std::thread> pool;
  for (uint32_t w = 1; w < workers; ++w) pool.emplace_back(run, w);
  run(0);
  for (auto& t : pool) t.join();
  for (uint32_t w = 0; w < workers; ++w)
    if (codes[w] != 0) throw Error(codes[w], errors[w]);
}

void store_bin(void* bins, bool wide, uint64_t index, uint32_t bin) {
  if (wide) static_cast<uint16_t*>(bins)[index] = uint16_t(bin);
  else static_cast<uint8_t*>(bins)[index] = uint8_t(bin);
}

}  // namespace

void quantize_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                    uint64_t rs, uint64_t cs, uint32_t max_bins, uint32_t n_threads, void* bins,
                    uint8_t* missing, float* boundaries, uint64_t* boundary_offset,
                    uint32_t* boundary_count, uint32_t* bin_count, uint64_t* missing_count) {
  const View v{static_cast<const uint8_t*>(data), scalar_type, rows, features, rs, cs};
  validate(v, max_bins);
  const bool wide = max_bins > 256;
  std::vector<std::vector<float>> per_feature(features);
  parallel_features(features, n_threads, [&](uint32_t f) {
    std::vector<float> column(rows);
    std::vector<float> sorted;
    sorted.reserve(rows);
    uint64_t n_missing = 0;
    for (uint64_t r = 0; r < rows; ++r) {
      const float x = read_value(v, r, f);
      column[r] = x;
      if (std::isnan(x)) ++n_missing;
      else sorted.push_back(x);
    }
    std::vector<float>& b = per_feature[f];
    if (!sorted.empty()) {
      std::sort(sorted.begin(), sorted.end());
      const uint64_t m = sorted.size();
      const uint64_t desired = std::min<uint64_t>(max_bins, m);
      const float maximum = sorted.back();
      for (uint64_t part = 1; part < desired; ++part) {
        const float c = sorted[quantile_rank(part, m, desired)];
        if (c < maximum && (b.empty() || c > b.back())) b.push_back(c);
      }
    }
    missing_count[f] = n_missing;
    boundary_count[f] = uint32_t(b.size());
    bin_count[f] = uint32_t(b.size() + 1);
    for (uint64_t r = 0; r < rows; ++r) {
      const float x = column[r];
      const bool miss = std::isnan(x);
      const uint32_t bin =
          miss ? 0u : uint32_t(std::lower_bound(b.begin(), b.end(), x) - b.begin());
      const uint64_t out = uint64_t(f) * rows + r;
      missing[out] = miss ? 1 : 0;
      store_bin(bins, wide, out, bin);
    }
  });
  uint64_t offset = 0;
  for (uint32_t f = 0; f < features; ++f) {
    boundary_offset[f] = offset;
    std::copy(per_feature[f].begin(), per_feature[f].end(), boundaries + offset);
    offset += per_feature[f].size();
  }
}

void transform_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                     uint64_t rs, uint64_t cs, uint32_t max_bins, const float* boundaries,
                     const uint64_t* boundary_offset, const uint32_t* boundary_count,
                     uint32_t n_threads, void* bins, uint8_t* missing) {
  const View v{static_cast<const uint8_t*>(data), scalar_type, rows, features, rs, cs};
  validate(v, max_bins);
  const bool wide = max_bins > 256;
  parallel_features(features, n_threads, [&](uint32_t f) {
    const float* first = boundaries + boundary_offset[f];
    const float* last = first + boundary_count[f];
    for (uint64_t r = 0; r < rows; ++r) {
      const float x = read_value(v, r, f);
      const bool miss = std::isnan(x);
      const uint32_t bin = miss ? 0u : uint32_t(std::lower_bound(first, last, x) - first);
      const uint64_t out = uint64_t(f) * rows + r;
      missing[out] = miss ? 1 : 0;
      store_bin(bins, wide, out, bin);
    }
  });
}

}  // namespace mpsb
