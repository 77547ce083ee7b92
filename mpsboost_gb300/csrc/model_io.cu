// The native model file: version 1.4 of the reference's binary format, so models trained
// here load in the reference and the reference's models load here.
//
// Layout (little-endian; src/io/model_format.cpp, model_payload.cpp,
// model_format_internal.hpp:21-28 of the reference):
//   header  magic "MPSBMOD\0", u16 major = 1, u16 minor = 4, u32 kind (0 regression,
//           1 multiclass), u64 payload size, u64 FNV-1a 64 checksum of the payload
//   payload features u32, max_bins u32, base_score f64, learning_rate f64,
//           objective u32, objective_alpha f64, tweedie_variance_power f64 (minor >= 4),
//           boundary count u64, per feature {boundary offset u64, boundary count u32,
//           bin count u32, missing count u64 (minor >= 2)}, boundaries f32[],
//           tree count u32, per tree node count u32 and 40-byte nodes {feature, threshold,
//           left, right u32; leaf, gain f64; default_left u8 (minor >= 2); flags u8;
//           reserved zero bytes (6, or 7 before minor 2)}.
// Reading accepts minors 0-4 and applies the reference's validation (schema ranges and
// strictly increasing finite boundaries, reachable acyclic trees, finite values, split
// thresholds inside the feature's bins, zero reserved bytes, no trailing bytes); every
// violation is a TrainingError (DataError for the schema), as in the reference.
#include <fcntl.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "host_types.h"

using namespace mpsb;

namespace {

constexpr uint8_t kMagic[8] = {'M', 'P', 'S', 'B', 'M', 'O', 'D', 0};
constexpr uint16_t kMajor = 1, kMinor = 4;
constexpr uint32_t kRegressionKind = 0;
constexpr uint32_t kMulticlassKind = 1;
constexpr size_t kHeaderBytes = 32;

uint64_t fnv1a64(const uint8_t* p, size_t n) {
  uint64_t h = 14695981039346656037ull;
  for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 1099511628211ull;
  return h;
}

struct Writer {
  std::vector<uint8_t> out;
  template <class T>
  void u(T v) {
    for (size_t i = 0; i < sizeof(T); ++i) out.push_back(uint8_t((uint64_t(v) >> (8 * i)) & 0xFF));
  }
  void f64(double v) {
    uint64_t b;
    std::memcpy(&b, &v, 8);
    u(b);
  }
  void f32(float v) {
    uint32_t b;
    std::memcpy(&b, &v, 4);
    u(b);
  }
};

struct Reader {
  const uint8_t* p;
  size_t n, pos = 0;
  template <class T>
  T u(const char* what) {
    if (sizeof(T) > n - pos) throw TrainingError(std::string("Model data is truncated: ") + what);
    uint64_t v = 0;
    for (size_t i = 0; i < sizeof(T); ++i) v |= uint64_t(p[pos++]) << (8 * i);
    return T(v);
  }
  double f64(const char* what) {
    const uint64_t b = u<uint64_t>(what);
    double v;
    std::memcpy(&v, &b, 8);
    if (!std::isfinite(v)) throw TrainingError(std::string("Model floating-point field is not finite: ") + what);
    return v;
  }
  float f32(const char* what) {
    const uint32_t b = u<uint32_t>(what);
    float v;
    std::memcpy(&v, &b, 4);
    if (!std::isfinite(v)) throw TrainingError(std::string("Model floating-point field is not finite: ") + what);
    return v;
  }
};

// ValidateSchemaFields (binned_dataset_internal.cpp:50-88).
void validate_schema(const mpsb_cuda_model& m) {
  if (m.features == 0 || m.max_bins < 2 || m.max_bins > 65536)
    throw DataError("Binned schema feature count or max_bins is invalid");
  uint64_t expected = 0;
  for (uint32_t f = 0; f < m.features; ++f) {
    const uint32_t cnt = m.boundary_count[f], bins = m.bin_count[f];
    if (m.boundary_offset[f] != expected || bins == 0 || bins != cnt + 1 || bins > m.max_bins)
      throw DataError("Binned schema boundary range or bin count is invalid");
    const uint64_t end = expected + cnt;
    if (end > m.boundaries.size()) throw DataError("Binned schema boundary range is out of bounds");
    for (uint32_t i = 0; i < cnt; ++i) {
      const float v = m.boundaries[expected + i];
      if (!std::isfinite(v) || (i != 0 && v <= m.boundaries[expected + i - 1]))
        throw DataError("Binned schema feature boundaries must be finite and strictly increasing");
    }
    expected = end;
  }
  if (expected != m.boundaries.size()) throw DataError("Binned schema contains boundaries not referenced by a feature");
}

// ValidateTreeStructure (tree_structure.cpp:150-187) and the per-node checks of
// RegressionModel::Restore (trainer.cpp:284-317).
void validate_tree(const std::vector<mpsb_tree_node>& nodes, const mpsb_cuda_model& m) {
  if (m.features == 0 || nodes.empty() || nodes.size() >= 0xFFFFFFFFull)
    throw TrainingError("Model tree feature count or node count is invalid");
  std::vector<uint8_t> state(nodes.size(), 0);
  std::vector<std::pair<uint32_t, bool>> stack{{0u, false}};
  while (!stack.empty()) {  // iterative depth-first visit: 1 = on the path, 2 = done
    auto [i, leaving] = stack.back();
    stack.pop_back();
    if (leaving) {
      state[i] = 2;
      continue;
    }
    if (i >= nodes.size()) throw TrainingError("Model tree child index is out of bounds");
    if (state[i] == 1) throw TrainingError("Model tree structure contains a cycle");
    if (state[i] == 2) continue;
    state[i] = 1;
    const mpsb_tree_node& n = nodes[i];
    if (n.flags & 1) {
      if (n.flags != 1 || !std::isfinite(n.leaf_value)) throw TrainingError("Model tree leaf value is not finite");
      state[i] = 2;
      continue;
    }
    if (n.flags != 0 || n.feature_index >= m.features || !std::isfinite(n.gain) || n.gain <= 0.0 ||
        n.left_child == n.right_child)
      throw TrainingError("Model tree branch fields are invalid");
    stack.push_back({i, true});
    stack.push_back({n.right_child, false});
    stack.push_back({n.left_child, false});
  }
  for (uint8_t s : state)
    if (s == 0) throw TrainingError("Model tree contains unreachable nodes");
  for (const mpsb_tree_node& n : nodes) {
    if (!(n.flags & 1) && n.threshold_bin >= m.bin_count[n.feature_index] - 1)
      throw TrainingError("Model tree split threshold exceeds the feature bin range");
    if ((n.flags & 1) && !n.default_left) throw TrainingError("model leaf nodes must keep default_left true");
  }
}

// MulticlassModel::Restore (multiclass_trainer.cpp:151-194).
void validate_softmax(const mpsb_cuda_model& m) {
  const uint32_t K = m.class_count;
  if (K < 2 || m.base_scores.size() != K || m.class_labels.size() != K || m.trees.empty() ||
      m.trees.size() % K != 0 || !std::isfinite(m.learning_rate) || m.learning_rate <= 0.0 ||
      m.learning_rate > 1.0)
    throw TrainingError("softmax model metadata is invalid");
  for (uint32_t k = 0; k < K; ++k) {
    if (!std::isfinite(m.base_scores[k]) || !std::isfinite(m.class_labels[k]))
      throw TrainingError("softmax model class metadata is not finite");
    if (k > 0 && !(m.class_labels[k - 1] < m.class_labels[k]))
      throw TrainingError("softmax model class labels must be strictly increasing");
  }
  for (const auto& t : m.trees) validate_tree(t, m);
}

void validate_model(const mpsb_cuda_model& m) {
  if (m.class_count) return validate_softmax(m);
  if (!std::isfinite(m.base) || !std::isfinite(m.learning_rate) || m.learning_rate <= 0.0 ||
      m.learning_rate > 1.0 || m.trees.empty())
    throw TrainingError("Model base score, learning rate, or tree count is invalid");
  if (!std::isfinite(m.objective_alpha) || m.objective_alpha <= 0.0 || m.objective_alpha >= 1.0)
    throw TrainingError("model quantile alpha is invalid");
  if (!std::isfinite(m.tweedie_variance_power) || m.tweedie_variance_power <= 1.0 ||
      m.tweedie_variance_power >= 2.0)
    throw TrainingError("model tweedie variance power is invalid");
  if (m.objective > 4) throw TrainingError("model objective is unsupported");
  for (const auto& t : m.trees) validate_tree(t, m);
}

void write_schema_tail(Writer& w, const mpsb_cuda_model& m) {  // boundary count .. boundaries
  w.u(uint64_t(m.boundaries.size()));
  for (uint32_t f = 0; f < m.features; ++f) {
    w.u(m.boundary_offset[f]);
    w.u(m.boundary_count[f]);
    w.u(m.bin_count[f]);
    w.u(m.missing_count[f]);
  }
  for (float b : m.boundaries) w.f32(b);
}

std::vector<uint8_t> serialize(const mpsb_cuda_model& m) {
  if (!m.has_schema) throw TrainingError("the model holds no quantization schema; attach the training data's");
  validate_model(m);
  Writer w;
  if (m.class_count) {  // BuildPayload(MulticlassModel), model_payload.cpp
    w.u(m.class_count);
    w.f64(m.learning_rate);
    for (double v : m.base_scores) w.f64(v);
    for (double v : m.class_labels) w.f64(v);
    w.u(m.features);
    w.u(m.max_bins);
    write_schema_tail(w, m);
  } else {
    w.u(m.features);
    w.u(m.max_bins);
    w.f64(m.base);
    w.f64(m.learning_rate);
    w.u(m.objective);
    w.f64(m.objective_alpha);
    w.f64(m.tweedie_variance_power);
    write_schema_tail(w, m);
  }
  w.u(uint32_t(m.trees.size()));
  for (const auto& t : m.trees) {
    w.u(uint32_t(t.size()));
    for (const mpsb_tree_node& n : t) {
      w.u(n.feature_index);
      w.u(n.threshold_bin);
      w.u(n.left_child);
      w.u(n.right_child);
      w.f64(n.leaf_value);
      w.f64(n.gain);
      w.u(uint8_t(n.default_left ? 1 : 0));
      w.u(n.flags);
      for (int i = 0; i < 6; ++i) w.u(uint8_t(0));
    }
  }
  Writer h;
  for (uint8_t c : kMagic) h.u(c);
  h.u(kMajor);
  h.u(kMinor);
  h.u(m.class_count ? kMulticlassKind : kRegressionKind);
  h.u(uint64_t(w.out.size()));
  h.u(fnv1a64(w.out.data(), w.out.size()));
  h.out.insert(h.out.end(), w.out.begin(), w.out.end());
  return h.out;
}

// expect: -1 either kind, 0 the regression loader, 1 the multiclass loader.
mpsb_cuda_model* deserialize(const uint8_t* bytes, size_t size, int expect) {
  if (size < kHeaderBytes || std::memcmp(bytes, kMagic, 8) != 0)
    throw TrainingError("Model magic does not match or header is truncated");
  Reader hr{bytes + 8, size - 8};
  const uint16_t major = hr.u<uint16_t>("major");
  const uint16_t minor = hr.u<uint16_t>("minor");
  const uint32_t kind = hr.u<uint32_t>("model kind");
  const uint64_t payload = hr.u<uint64_t>("payload size");
  const uint64_t checksum = hr.u<uint64_t>("checksum");
  if (major != kMajor) throw TrainingError("Model major version is unsupported");
  if (expect == 0 && kind != kRegressionKind)
    throw TrainingError("model kind is incompatible with regression loader");
  if (expect == 1 && kind != kMulticlassKind)
    throw TrainingError("model kind is incompatible with multiclass loader");
  if (kind != kRegressionKind && kind != kMulticlassKind) throw TrainingError("model kind is unsupported");
  if (payload != size - kHeaderBytes) throw TrainingError("Model payload length does not match");
  const uint8_t* p = bytes + kHeaderBytes;
  if (fnv1a64(p, payload) != checksum) throw TrainingError("Model integrity check failed");
  Reader r{p, size_t(payload)};
  std::unique_ptr<mpsb_cuda_model> m(new mpsb_cuda_model);
  if (kind == kMulticlassKind) {  // ParseMulticlassPayload, model_payload.cpp
    if (minor < 3) throw TrainingError("multiclass model format is unsupported");
    m->class_count = r.u<uint32_t>("class_count");
    m->learning_rate = r.f64("learning_rate");
    if (m->class_count > payload / 16) throw TrainingError("softmax model metadata is invalid");
    m->base_scores.resize(m->class_count);
    for (auto& v : m->base_scores) v = r.f64("softmax base_score");
    m->class_labels.resize(m->class_count);
    for (auto& v : m->class_labels) v = r.f64("softmax class label");
    m->features = r.u<uint32_t>("features");
    m->max_bins = r.u<uint32_t>("max_bins");
  } else {
    m->features = r.u<uint32_t>("features");
    m->max_bins = r.u<uint32_t>("max_bins");
    m->base = r.f64("base_score");
    m->learning_rate = r.f64("learning_rate");
    if (minor >= 1) {
      m->objective = r.u<uint32_t>("objective");
      if (m->objective > 4) throw TrainingError("model objective is unsupported");
    }
    if (minor >= 4) {
      m->objective_alpha = r.f64("objective_alpha");
      m->tweedie_variance_power = r.f64("tweedie_variance_power");
    }
  }
  const uint64_t n_bounds = r.u<uint64_t>("boundary_count");
  if (n_bounds > payload / sizeof(float)) throw TrainingError("Model boundary_count exceeds the payload range");
  m->boundary_offset.resize(m->features);
  m->boundary_count.resize(m->features);
  m->bin_count.resize(m->features);
  m->missing_count.assign(m->features, 0);
  for (uint32_t f = 0; f < m->features; ++f) {
    m->boundary_offset[f] = r.u<uint64_t>("boundary_offset");
    m->boundary_count[f] = r.u<uint32_t>("feature boundary_count");
    m->bin_count[f] = r.u<uint32_t>("feature bin_count");
    if (minor >= 2) m->missing_count[f] = r.u<uint64_t>("feature missing_count");
  }
  m->boundaries.resize(size_t(n_bounds));
  for (auto& b : m->boundaries) b = r.f32("boundary");
  m->has_schema = true;
  validate_schema(*m);
  const uint32_t n_trees = r.u<uint32_t>("tree_count");
  if (n_trees == 0 || n_trees > payload / 41) throw TrainingError("Model tree count is invalid");
  m->trees.resize(n_trees);
  for (auto& t : m->trees) {
    const uint32_t n_nodes = r.u<uint32_t>("node_count");
    if (n_nodes == 0 || n_nodes > payload / 41) throw TrainingError("Model node count is invalid");
    t.resize(n_nodes);
    for (mpsb_tree_node& n : t) {
      n.feature_index = r.u<uint32_t>("feature_index");
      n.threshold_bin = r.u<uint32_t>("threshold_bin");
      n.left_child = r.u<uint32_t>("left_child");
      n.right_child = r.u<uint32_t>("right_child");
      n.leaf_value = r.f64("leaf_value");
      n.gain = r.f64("gain");
      n.default_left = 1;
      if (minor >= 2) {
        const uint8_t dl = r.u<uint8_t>("default_left");
        if (dl > 1) throw TrainingError("model default_left must be 0 or 1");
        n.default_left = dl;
      }
      n.flags = r.u<uint8_t>("flags");
      const int reserved = minor >= 2 ? 6 : 7;
      for (int i = 0; i < reserved; ++i)
        if (r.u<uint8_t>("node reserved") != 0) throw TrainingError("Model node reserved fields must be zero");
      std::memset(n.reserved, 0, sizeof n.reserved);
    }
  }
  if (r.pos != r.n) throw TrainingError("Model contains unrecognized trailing bytes");
  m->n_trees = n_trees;
  validate_model(*m);
  return m.release();
}

std::string errno_message(const char* stage) { return std::string(stage) + ": " + std::strerror(errno); }

// Write to a temporary file in the target's directory, flush it to disk and rename it
// over the target, so a reader never sees a partial model.
void write_file(const std::vector<uint8_t>& bytes, const std::string& path) {
  if (path.empty()) throw TrainingError("Model save path must not be empty");
  const size_t slash = path.find_last_of('/');
  const std::string dir = slash == std::string::npos ? "." : (slash == 0 ? "/" : path.substr(0, slash));
  const std::string name = slash == std::string::npos ? path : path.substr(slash + 1);
  std::string pattern = dir + "/." + name + ".mpsboost-XXXXXX";
  std::vector<char> tmpl(pattern.begin(), pattern.end());
  tmpl.push_back('\0');
  const int fd = ::mkstemp(tmpl.data());
  if (fd < 0) throw TrainingError(errno_message("Failed to create temporary model file"));
  size_t done = 0;
  while (done < bytes.size()) {
    const ssize_t k = ::write(fd, bytes.data() + done, bytes.size() - done);
    if (k <= 0) {
      ::close(fd);
      ::unlink(tmpl.data());
      throw TrainingError(errno_message("Failed to write temporary model file"));
    }
    done += size_t(k);
  }
  if (::fsync(fd) != 0 || ::close(fd) != 0) {
    ::unlink(tmpl.data());
    throw TrainingError(errno_message("Failed to synchronize temporary model file"));
  }
  if (::rename(tmpl.data(), path.c_str()) != 0) {
    ::unlink(tmpl.data());
    throw TrainingError(errno_message("Failed to atomically replace model file"));
  }
}

std::vector<uint8_t> read_file(const std::string& path) {
  if (path.empty()) throw TrainingError("Model load path must not be empty");
  const int fd = ::open(path.c_str(), O_RDONLY);
  if (fd < 0) throw TrainingError(errno_message("Failed to open model file"));
  std::vector<uint8_t> bytes;
  uint8_t buf[1 << 16];
  for (;;) {
    const ssize_t k = ::read(fd, buf, sizeof buf);
    if (k < 0) {
      ::close(fd);
      throw TrainingError(errno_message("Failed to read model file"));
    }
    if (k == 0) break;
    bytes.insert(bytes.end(), buf, buf + k);
  }
  ::close(fd);
  return bytes;
}

}  // namespace

extern "C" {

int mpsb_cuda_model_set_schema(mpsb_cuda_model* m, uint32_t features, uint32_t max_bins,
                               const float* boundaries, uint64_t n_boundaries,
                               const uint64_t* boundary_offset, const uint32_t* boundary_count,
                               const uint32_t* bin_count, const uint64_t* missing_count) {
  return guard([&] {
    if (!m || !boundary_offset || !boundary_count || !bin_count || (n_boundaries && !boundaries))
      throw TrainingError("null argument");
    mpsb_cuda_model s;
    s.features = features;
    s.max_bins = max_bins;
    s.boundaries.assign(boundaries, boundaries + n_boundaries);
    s.boundary_offset.assign(boundary_offset, boundary_offset + features);
    s.boundary_count.assign(boundary_count, boundary_count + features);
    s.bin_count.assign(bin_count, bin_count + features);
    s.missing_count.assign(features, 0);
    if (missing_count) s.missing_count.assign(missing_count, missing_count + features);
    validate_schema(s);
    m->features = s.features;
    m->max_bins = s.max_bins;
    m->boundaries = std::move(s.boundaries);
    m->boundary_offset = std::move(s.boundary_offset);
    m->boundary_count = std::move(s.boundary_count);
    m->bin_count = std::move(s.bin_count);
    m->missing_count = std::move(s.missing_count);
    m->has_schema = true;
  });
}

int mpsb_cuda_model_set_objective(mpsb_cuda_model* m, uint32_t objective, double alpha,
                                  double variance_power) {
  return guard([&] {
    if (!m) throw TrainingError("null argument");
    if (objective > 4) throw TrainingError("model objective is unsupported");
    m->objective = objective;
    m->objective_alpha = alpha;
    m->tweedie_variance_power = variance_power;
  });
}

int mpsb_cuda_model_get_objective(const mpsb_cuda_model* m, uint32_t* objective, double* alpha,
                                  double* variance_power) {
  return guard([&] {
    if (!m) throw TrainingError("null argument");
    if (objective) *objective = m->objective;
    if (alpha) *alpha = m->objective_alpha;
    if (variance_power) *variance_power = m->tweedie_variance_power;
  });
}

int mpsb_cuda_model_get_schema(const mpsb_cuda_model* m, uint32_t* features, uint32_t* max_bins,
                               uint64_t* n_boundaries, float* boundaries, uint64_t* boundary_offset,
                               uint32_t* boundary_count, uint32_t* bin_count,
                               uint64_t* missing_count) {
  return guard([&] {
    if (!m) throw TrainingError("null argument");
    if (!m->has_schema) throw TrainingError("the model holds no quantization schema");
    if (features) *features = m->features;
    if (max_bins) *max_bins = m->max_bins;
    if (n_boundaries) *n_boundaries = m->boundaries.size();
    if (boundaries) std::memcpy(boundaries, m->boundaries.data(), m->boundaries.size() * sizeof(float));
    if (boundary_offset) std::memcpy(boundary_offset, m->boundary_offset.data(), m->features * 8);
    if (boundary_count) std::memcpy(boundary_count, m->boundary_count.data(), m->features * 4);
    if (bin_count) std::memcpy(bin_count, m->bin_count.data(), m->features * 4);
    if (missing_count) std::memcpy(missing_count, m->missing_count.data(), m->features * 8);
  });
}

int mpsb_cuda_model_serialize(const mpsb_cuda_model* m, uint8_t* out, uint64_t capacity,
                              uint64_t* size) {
  return guard([&] {
    if (!m || !size) throw TrainingError("null argument");
    const std::vector<uint8_t> bytes = serialize(*m);
    *size = bytes.size();
    if (out) {
      if (capacity < bytes.size()) throw TrainingError("model serialization buffer is too small");
      std::memcpy(out, bytes.data(), bytes.size());
    }
  });
}

int mpsb_cuda_model_deserialize(const uint8_t* data, uint64_t size, int kind,
                                mpsb_cuda_model** out) {
  return guard([&] {
    if (!data || !out) throw TrainingError("null argument");
    *out = deserialize(data, size_t(size), kind);
  });
}

int mpsb_cuda_model_save(const mpsb_cuda_model* m, const char* path) {
  return guard([&] {
    if (!m || !path) throw TrainingError("null argument");
    write_file(serialize(*m), path);
  });
}

int mpsb_cuda_model_load(const char* path, int kind, mpsb_cuda_model** out) {
  return guard([&] {
    if (!path || !out) throw TrainingError("null argument");
    const std::vector<uint8_t> bytes = read_file(path);
    *out = deserialize(bytes.data(), bytes.size(), kind);
  });
}

}  // extern "C"
