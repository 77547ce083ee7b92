// Device-side data structures and exact arithmetic shared by the sm_103a kernels.
//
// FP64 expressions that restate the reference's objective math use explicit
// round-to-nearest intrinsics (__dadd_rn, __dmul_rn, __ddiv_rn) so the compiler can never
// fuse a multiply and an add: each operation rounds exactly once, as in the reference
// C++ (src/core/objective.cpp:264-356) compiled without contraction.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mpsb {

constexpr int kSlots = 256;          // histogram slots per feature
constexpr int kMissingSlot = 255;    // bin value of a missing row (features with missing)
constexpr int kBlockFeatures = 32;   // features per column block of the bin matrix
constexpr uint32_t kItemRowsMax = 65536;  // rows of one histogram work item (limb bound)
constexpr uint32_t kPartChunk = 4096;     // rows per partition chunk
constexpr uint32_t kApplyChunk = 4096;    // rows per leaf-application chunk

// kModeFixedG: fixed point, gradient limbs only (a root build whose count and hessian
// histograms are restored from the fit's first round).
// kModeFixedCG: fixed point, count and gradient limbs; every row's hessian is the same
// quantized unit (unweighted squared error and quantile: h = 1), so a cell's hessian
// sum is its count times that unit, exactly.
enum : int { kModeFixed = 0, kModeFloat = 1, kModeFixedG = 2, kModeFixedCG = 3 };

// Device status bits (ORed into TrainerState::error).
enum : uint32_t {
  kErrCountMismatch = 1u << 0,   // histogram count != node count (tree_split.cpp:179-181)
  kErrNonFinite = 1u << 1,       // non-finite statistic, gain or leaf value
  kErrHessian = 1u << 2,         // negative Hessian sum
  kErrSubtraction = 1u << 3,     // child bin exceeds parent bin (tree_histogram.cpp:44-60)
  kErrPartition = 1u << 4,       // partition counts differ (tree_split.cpp:286-289)
  kErrMissing = 1u << 5,         // missing stats exceed parent (tree_split.cpp:186-189)
  kErrCapacity = 1u << 6,        // an internal table overflowed
  kErrGradient = 1u << 7,        // invalid label / prediction / weight / gradient
  kErrPrefix = 1u << 8,          // prefix exceeded the non-missing parent (tree_split.cpp:212-214)
  kErrRootCache = 1u << 9,       // the hessian scale of a reused root histogram changed
  kErrLeafQueue = 1u << 10,      // leaf-wise active queue beyond max_active_leaves
  kErrCopy = 1u << 11,           // a tensor copy did not complete within its time limit
                                 // (tree_leafwise.cpp:80-83, 130-134)
};

// Tree parameters resolved on the host (tree.hpp:47-72, tree_structure.cpp:54-62).
struct TreeParams {
  uint64_t min_samples_leaf;
  double min_child_weight;
  double reg_lambda;
  double reg_alpha;
  double max_delta_step;
  double gamma;
  double min_gain_to_split;
  double learning_rate;
  uint32_t max_depth;
  uint32_t max_leaves;  // effective
  uint32_t split_strategy;
  uint32_t random_seed;
  uint32_t has_monotonic;
  uint32_t n_groups;
  uint32_t path_words;  // ceil(features / 32)
  uint32_t objective;
  double objective_alpha;
  double tweedie_variance_power;
  // The split scan's FP32 screen constants, derived on the host (set_screen_constants):
  // computed in the kernel, the double-to-float conversions and FP64 compares were
  // re-evaluated at their uses inside the candidate loop, on the narrow FP64 pipe.
  float screen_lambda;                 // float(reg_lambda)
  float screen_mcw_lo, screen_mcw_hi;  // float(min_child_weight) x (1 - 3e-6), x (1 + 3e-6)
  uint32_t screen_mcw_on;              // min_child_weight > 0
  uint32_t screen_params;              // split_strategy 0, reg_alpha 0, reg_lambda > 0
};

// Fills the screen constants of a TreeParams from its FP64 fields (IEEE float conversion
// and multiplication: the same values the device computes).
inline void set_screen_constants(TreeParams& p) {
  const float mcw32 = float(p.min_child_weight);
  p.screen_lambda = float(p.reg_lambda);
  p.screen_mcw_lo = mcw32 * (1.0f - 3e-6f);
  p.screen_mcw_hi = mcw32 * (1.0f + 3e-6f);
  p.screen_mcw_on = p.min_child_weight > 0.0 ? 1u : 0u;
  p.screen_params = (p.split_strategy == 0 && p.reg_alpha == 0.0 && p.reg_lambda > 0.0) ? 1u : 0u;
}

// One node of a depth level. Statistics are exact int64 (fixed mode; g/h hold the FP64
// images q * 2^-k) or FP64 (float mode).
struct NodeRec {
  uint32_t seg_off;
  uint32_t seg_cnt;
  uint32_t node_index;  // index in the tree's flat node array
  uint32_t slot;        // histogram slot
  uint64_t count;
  long long qg, qh;
  double g, h;
  double lo, hi;        // monotone bounds of the node's leaf value
  uint32_t tree;
  uint32_t depth;
  // 0: the slot holds the node's histogram. k + 1: the slot still holds the parent's, and
  // the level's first split-scan launch subtracts the built sibling's (slot k) from it,
  // feature by feature as it scans them, and writes the difference back.
  uint32_t sub_from;
};

// Best split of a node or of a (node, feature chunk); the SplitCandidate of
// tree_internal.hpp:32-45 with exact statistics.
struct SplitRec {
  double gain;
  uint32_t valid, feature, threshold, default_left;
  uint64_t lcount, rcount;
  long long lqg, lqh, rqg, rqh;
  double lg, lh, rg, rh;
  double ll, lu, rl, ru;
};
static_assert(sizeof(SplitRec) % 8 == 0 && sizeof(SplitRec) / 8 <= 32,
              "a warp copies a SplitRec one 8-byte word per lane");

// An active leaf of leaf-wise growth (ActiveNode, tree_internal.hpp:44-53): its node, the
// row buffer holding its segment, and its best split once scanned.
struct LeafActive {
  NodeRec node;
  SplitRec best;
  uint32_t parity;
  uint32_t scanned;
};

// Output tree node, layout of mpsb_tree_node.
struct TreeNodeOut {
  uint32_t feature_index, threshold_bin, left_child, right_child;
  double leaf_value, gain;
  uint8_t default_left, flags, reserved[6];
};

// A segment whose rows receive a leaf update: constant leaf, or (split != 0) routed by
// the parent's split to its two children (last level: no partition is needed).
struct LeafSeg {
  uint32_t tree, parity, seg_off, seg_cnt;
  uint32_t split, feature, threshold, default_left;
  double value, left_value, right_value;
};

// Histogram build entry: one node whose histogram is accumulated from its rows.
struct BuildEntry {
  uint32_t tree, parity, seg_off, seg_cnt, slot, pad;
};

// Sibling subtraction: slot_sibling := slot_parent - slot_built (in place on the parent).
struct SubEntry {
  uint32_t parent_slot, built_slot;
};

// Accepted split whose rows are partitioned into the next level's buffer.
struct PartEntry {
  uint32_t tree, parity, seg_off, seg_cnt;
  uint32_t feature, threshold, default_left, lcount;
};

// Per-tree round state.
struct TreeState {
  uint32_t max_abs_g_bits;  // float bits of max |g| (non-negative floats order as uints)
  uint32_t max_h_bits;
  int32_t kg, kh;           // fixed-point exponents
  double inv_g, inv_h;      // 2^-kg, 2^-kh
  uint32_t n_tree_nodes;
  uint32_t leaf_count;
};

// Whole-trainer control block (device memory).
struct Control {
  uint32_t error;          // kErr* bits
  uint32_t n_nodes;        // nodes in the current level (all trees)
  uint32_t n_build;        // build entries of the current level
  uint32_t n_sub;          // subtraction pairs of the current level
  uint32_t n_part;         // partition entries of the current level
  uint32_t n_leafseg;      // leaf segments of the current round
  uint32_t hist_items;     // build chunks x feature blocks
  uint32_t hist_counter;   // work-stealing counter of the histogram kernel
  uint32_t part_chunks;
  uint32_t leaf_chunks;
  uint32_t free_top;       // histogram-slot free stack
  uint32_t split_items;    // nodes x feature chunks
  uint32_t item_rows;      // rows per histogram work item of the current level
  unsigned long long cells;       // cumulative row x feature cells built (accounting)
  unsigned long long rows_built;
  unsigned long long rows_partitioned;  // rows routed by partitions (accounting)
};

// ---------------------------------------------------------------------------------
// Exact FP64 objective math (objective.cpp:264-356, tree_structure.cpp:72-87).
// Each returns false where the reference throws TrainingError.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool soft_threshold(double g, double alpha, double* out) {
  if (!isfinite(g)) return false;
  const double magnitude = __dadd_rn(fabs(g), -alpha);
  *out = magnitude <= 0.0 ? 0.0 : copysign(magnitude, g);
  return true;
}

__device__ __forceinline__ bool node_score(double g, double h, double lambda, double alpha,
                                           double* out) {
  double rg;
  if (!soft_threshold(g, alpha, &rg)) return false;
  if (!isfinite(h) || h < 0.0) return false;
  const double d = __dadd_rn(h, lambda);
  if (!isfinite(d) || d <= 0.0) return false;
  *out = __ddiv_rn(__dmul_rn(rg, rg), d);
  return isfinite(*out);
}

__device__ __forceinline__ bool leaf_weight(double g, double h, const TreeParams& p,
                                            double* out) {
  double rg;
  if (!soft_threshold(g, p.reg_alpha, &rg)) return false;
  if (!isfinite(h) || h < 0.0) return false;
  const double d = __dadd_rn(h, p.reg_lambda);
  if (!isfinite(d) || d <= 0.0) return false;
  double w = __ddiv_rn(-rg, d);
  if (p.max_delta_step != 0.0) w = fmax(-p.max_delta_step, fmin(p.max_delta_step, w));
  *out = w;
  return isfinite(w);
}

__device__ __forceinline__ double clamp_bounds(double v, double lo, double hi) {
  return v < lo ? lo : (hi < v ? hi : v);  // std::clamp(v, lo, hi)
}

__device__ __forceinline__ bool split_gain(double lg, double lh, double rg, double rh,
                                           const TreeParams& p, double* out) {
  if (!isfinite(lh) || !isfinite(rh) || lh <= 0.0 || rh <= 0.0) return false;
  const double pg = __dadd_rn(lg, rg), ph = __dadd_rn(lh, rh);
  if (!isfinite(pg) || !isfinite(ph)) return false;
  double sl, sr, sp;
  if (!node_score(lg, lh, p.reg_lambda, p.reg_alpha, &sl)) return false;
  if (!node_score(rg, rh, p.reg_lambda, p.reg_alpha, &sr)) return false;
  if (!node_score(pg, ph, p.reg_lambda, p.reg_alpha, &sp)) return false;
  const double gain = __dadd_rn(__dmul_rn(0.5, __dadd_rn(__dadd_rn(sl, sr), -sp)), -p.gamma);
  *out = gain;
  return isfinite(gain);
}

// StableRandomThreshold (tree_split.cpp:14-29).
// Not inlined: its 64-bit remainder is a long subroutine that must not be speculated
// into scans that use no random thresholds.
static __device__ __noinline__ uint32_t stable_random_threshold(uint32_t seed, uint32_t feature,
                                                            uint32_t node, uint32_t depth,
                                                            uint32_t candidates) {
  unsigned long long v = seed;
  v ^= (unsigned long long)feature + 0x9E3779B97F4A7C15ULL;
  v *= 0xBF58476D1CE4E5B9ULL;
  v ^= ((unsigned long long)node << 32) | depth;
  v *= 0x94D049BB133111EBULL;
  v ^= v >> 31;
  return (uint32_t)(v % candidates);
}

// IEEE-754 conversions on the integer pipe. sm_103 runs FP64 arithmetic and 64-bit
// conversions on a narrow FP64 pipe; these give the round-to-nearest-even results of the
// standard (the bit patterns of a correctly rounded conversion) with 32/64-bit integer
// instructions only.

// Round-to-nearest-even of m * 2^-s for s in [1, 63]: the shifted value, possibly carrying
// one bit past its width.
__device__ __forceinline__ unsigned long long rne_shift(unsigned long long m, int s) {
  const unsigned long long q = m >> s;
  const unsigned long long rem = m & ((1ull << s) - 1ull);
  const unsigned long long half = 1ull << (s - 1);
  return q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
}

// (float)x, correctly rounded: one hardware conversion, which on sm_103 issues to the
// FP32 (FMA-lite) pipe, not the narrow FP64 pipe that takes the 64-bit-source
// conversions (ncu pipe counters of a conversion loop: about three instructions per
// conversion, none on the FP64 pipe).
__device__ __forceinline__ float u32_to_f32_rn(uint32_t x) { return __uint2float_rn(x); }

// (float)q, correctly rounded.
__device__ __forceinline__ float s64_to_f32_rn(long long q) {
  if (q == 0) return 0.0f;
  const uint32_t sign = q < 0 ? 0x80000000u : 0u;
  const unsigned long long a = q < 0 ? 0ull - (unsigned long long)q : (unsigned long long)q;
  int e = 63 - __clzll((long long)a);  // position of the leading bit
  unsigned long long m;
  if (e <= 23) {
    m = a << (23 - e);
  } else {
    m = rne_shift(a, e - 23);
    if (m == (1ull << 24)) {
      m >>= 1;
      ++e;
    }
  }
  return __uint_as_float(sign | (uint32_t(e + 127) << 23) | (uint32_t(m) & 0x7FFFFFu));
}

// True when the double is neither infinite nor NaN.
__device__ __forceinline__ bool f64_finite(double x) {
  return ((__double2hiint(x) >> 20) & 0x7FF) != 0x7FF;
}

// (float)x, correctly rounded (overflow to infinity, underflow through the subnormals).
__device__ __forceinline__ float f64_to_f32_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t sign = uint32_t(b >> 32) & 0x80000000u;
  const int e = int((b >> 52) & 0x7FF);
  const unsigned long long frac = b & ((1ull << 52) - 1ull);
  if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (frac ? 0x400000u : 0u));
  if (e == 0) return __uint_as_float(sign);  // |x| < 2^-1022: below half the least float
  const int E = e - 1023;
  const unsigned long long m = frac | (1ull << 52);
  if (E > 127) return __uint_as_float(sign | 0x7F800000u);
  if (E >= -126) {
    unsigned long long q = rne_shift(m, 29);
    int ee = E;
    if (q == (1ull << 24)) {
      q >>= 1;
      ++ee;
    }
    if (ee > 127) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | (uint32_t(ee + 127) << 23) | (uint32_t(q) & 0x7FFFFFu));
  }
  // Subnormal result: m * 2^(E-52) in units of 2^-149 is m * 2^(E+97).
  const int s = -E - 97;  // >= 30
  if (s > 53) return __uint_as_float(sign);  // below a quarter of the least subnormal
  return __uint_as_float(sign | uint32_t(rne_shift(m, s)));  // a carry gives 2^-126 exactly
}

// round_half_even(x * 2^k) for a finite float x, exactly, with integer arithmetic only.
// Equals llrint(ldexp((double)x, k)) whenever the result fits in int64 (the scale rule
// guarantees |result| < 2^62).
__device__ __forceinline__ long long quantize_f32(float x, int k) {
  const uint32_t bits = __float_as_uint(x);
  const uint32_t e = (bits >> 23) & 0xFFu;
  uint32_t mant = bits & 0x7FFFFFu;
  int exp2;
  if (e == 0) {
    exp2 = -149;
  } else {
    mant |= 0x800000u;
    exp2 = (int)e - 150;
  }
  const int shift = exp2 + k;
  unsigned long long q;
  if (shift >= 0) {
    q = (unsigned long long)mant << shift;
  } else if (shift < -25) {
    q = 0;  // |x * 2^k| < 2^24 * 2^-26 = 1/4
  } else {
    const int s = -shift;
    q = mant >> s;
    const uint32_t rem = mant & ((1u << s) - 1u);
    const uint32_t half = 1u << (s - 1);
    if (rem > half || (rem == half && (q & 1ull))) ++q;
  }
  return (bits >> 31) ? -(long long)q : (long long)q;
}

__device__ __forceinline__ double q_image(long long q, double inv) {
  return __dmul_rn(__ll2double_rn(q), inv);
}

// Total order of split candidates: IsBetterSplit (tree_split.cpp:31-45) with the missing
// direction tried first (default_left = true) winning exact ties.
__device__ __forceinline__ bool better_split(const SplitRec& a, const SplitRec& b) {
  if (!a.valid) return false;
  if (!b.valid) return true;
  if (a.gain != b.gain) return a.gain > b.gain;
  if (a.feature != b.feature) return a.feature < b.feature;
  if (a.threshold != b.threshold) return a.threshold < b.threshold;
  return a.default_left && !b.default_left;
}

}  // namespace mpsb
