// Host-side error type carrying an mpsb_cuda.h error code.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>

namespace mpsb {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
struct TrainingError : Error {
  explicit TrainingError(const std::string& m) : Error(1, m) {}
};
struct DataError : Error {
  explicit DataError(const std::string& m) : Error(2, m) {}
};
struct BackendError : Error {
  explicit BackendError(const std::string& m) : Error(3, m) {}
};
struct UnsupportedError : Error {
  explicit UnsupportedError(const std::string& m) : Error(4, m) {}
};

void quantize_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                    uint64_t rs, uint64_t cs, uint32_t max_bins, uint32_t n_threads, void* bins,
                    uint8_t* missing, float* boundaries, uint64_t* boundary_offset,
                    uint32_t* boundary_count, uint32_t* bin_count, uint64_t* missing_count);
void transform_dense(const void* data, int scalar_type, uint64_t rows, uint32_t features,
                     uint64_t rs, uint64_t cs, uint32_t max_bins, const float* boundaries,
                     const uint64_t* boundary_offset, const uint32_t* boundary_count,
                     uint32_t n_threads, void* bins, uint8_t* missing);

}  // namespace mpsb
