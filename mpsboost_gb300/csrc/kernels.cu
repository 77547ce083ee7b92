// Training-loop kernels for sm_103a (everything except the histogram build).
//
//   gradients      ComputeObjectiveGradients + ApplySampleWeights (trainer.cpp:178-216),
//                  FP64 math rounded once to FP32 pairs, plus per-tree max|g| / max h for
//                  the fixed-point scales.
//   round_setup    fixed-point exponents, root node, level-0 build list.
//   root_cache     the roots' count and hessian histograms kept from a fit's first round
//                  (objectives whose hessian does not depend on the prediction).
//   root_stats     root statistics from the root histogram; root leaf value
//                  (TreeTrainingAccess::Create, tree_structure.cpp:104-116).
//   subtract       SubtractHistograms (tree_histogram.cpp:16-66): exact int64 in fixed
//                  mode, FP64 with the Hessian clamp in float mode.
//   split_scan     FindBestSplit (tree_split.cpp:142-234): one warp per (node, feature),
//                  warp-shuffle prefix over the 256 slots, FP64 gains with both missing
//                  directions, random threshold, monotone and interaction rules.
//   finalize       the per-level bookkeeping of TrainLevelWiseRegressionTree
//                  (tree.cpp:67-145): acceptance under max_leaves, ApplySplit
//                  (tree_structure.cpp:118-148), smaller-child selection, next level.
//   partition      PrepareSplitRows' stable partition (tree_split.cpp:273-289) as a
//                  ballot/popc compaction: count, per-node scan, scatter.
//   apply_leaves   predictions += lr * leaf (trainer.cpp:256-262) from the final row
//                  segments: no tree traversal.
#include <algorithm>
#include <cfloat>
#include <type_traits>

#include "device.cuh"
#include "kernels.h"

namespace mpsb {
namespace {

__device__ __forceinline__ void raise(Control* ctl, uint32_t bits) { atomicOr(&ctl->error, bits); }

__device__ __forceinline__ uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

// Rows per histogram work item for a level that builds `rows` rows: about per_sm (default
// three) items per SM, a multiple of 512, within [4096, kItemRowsMax]. Where the
// kItemRowsMax cap forces more items, their number is raised to the next multiple of the
// SM count, so that the persistent CTAs end the level together.
__device__ __forceinline__ uint32_t adaptive_item_rows(uint64_t rows, uint32_t nfb, uint32_t sms,
                                                      uint32_t per_sm) {
  const uint64_t n_sm = sms ? sms : 152;
  uint64_t target = n_sm * (per_sm ? per_sm : 3);
  const uint64_t min_items = (rows * nfb + kItemRowsMax - 1) / kItemRowsMax;
  if (target < min_items) target = (min_items + n_sm - 1) / n_sm * n_sm;
  uint64_t per = (rows * nfb + target - 1) / target;
  per = (per + 511) / 512 * 512;
  if (per < 4096) per = 4096;
  if (per > kItemRowsMax) per = kItemRowsMax;
  return uint32_t(per);
}

// Exponent e with x < 2^e (frexp convention) of a positive finite float.
__device__ __forceinline__ int exponent_above(float x) {
  int e;
  frexpf(x, &e);
  return e;
}

// Block-wide exclusive scan of N values per thread. `sh` holds >= 33*N words.
template <int N>
__device__ void block_scan(uint32_t (&v)[N], uint32_t (&total)[N], uint32_t* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  uint32_t incl[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    uint32_t x = v[k];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    incl[k] = x;
    if (lane == 31) sh[warp * N + k] = x;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      uint32_t x = lane < nwarps ? sh[lane * N + k] : 0u;
      const uint32_t own = x;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
      }
      if (lane < nwarps) sh[lane * N + k] = x - own;
      if (lane == 31) sh[32 * N + k] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) {
    total[k] = sh[32 * N + k];
    v[k] = sh[warp * N + k] + incl[k] - v[k];
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------------
// Round begin / gradients / setup
// ------------------------------------------------------------------------------------
__global__ void round_begin_kernel(TrainerDev a) {
  for (uint32_t i = threadIdx.x; i < a.n_slots; i += blockDim.x) a.free_stack[i] = a.n_slots - 1 - i;
  for (uint32_t t = threadIdx.x; t < a.n_trees; t += blockDim.x) {
    a.trees[t].max_abs_g_bits = 0;
    a.trees[t].max_h_bits = 0;
    a.trees[t].n_tree_nodes = 1;
    a.trees[t].leaf_count = 1;
  }
  if (threadIdx.x == 0) {
    a.ctl->free_top = a.n_slots;
    a.ctl->n_leafseg = 0;
    a.ctl->leaf_chunks = 0;
    a.leaf_prefix[0] = 0;
  }
}

__device__ __forceinline__ double logistic_probability(double m) {  // objective.cpp:309-317
  if (m >= 0.0) {
    const double e = exp(-m);
    return __ddiv_rn(1.0, __dadd_rn(1.0, e));
  }
  const double e = exp(m);
  return __ddiv_rn(e, __dadd_rn(1.0, e));
}

// Objective gradient of one row (objective.cpp:290-429). Returns false on a reference
// TrainingError condition. Finiteness tests read the exponent bits (integer pipe); the
// FP64 pipe does only the arithmetic the reference rounds.
__device__ __forceinline__ bool objective_pair(uint32_t objective, double y, double p,
                                               const TreeParams& prm, double* g, double* h) {
  if (!f64_finite(y) || !f64_finite(p)) return false;
  switch (objective) {
    case 0:
      *g = __dadd_rn(p, -y);
      *h = 1.0;
      return f64_finite(*g);
    case 1: {
      if (y != 0.0 && y != 1.0) return false;
      const double prob = logistic_probability(p);
      *g = __dadd_rn(prob, -y);
      *h = __dmul_rn(prob, __dadd_rn(1.0, -prob));
      return isfinite(*g) && isfinite(*h) && *h >= 0.0;
    }
    case 2:
      *g = p < y ? -prm.objective_alpha : __dadd_rn(1.0, -prm.objective_alpha);
      *h = 1.0;
      return true;
    case 3: {
      if (y < 0.0 || p > 709.0) return false;
      const double mean = exp(p);
      *g = __dadd_rn(mean, -y);
      *h = mean;
      return isfinite(*g) && isfinite(*h) && *h > 0.0;
    }
    case 4: {
      const double rho = prm.tweedie_variance_power;
      const double a1 = __dmul_rn(__dadd_rn(2.0, -rho), p);
      const double a2 = __dmul_rn(__dadd_rn(1.0, -rho), p);
      if (y < 0.0 || a1 > 709.0 || a2 > 709.0) return false;
      const double first = exp(a1), second = exp(a2);
      *g = __dadd_rn(first, -__dmul_rn(y, second));
      *h = __dadd_rn(__dmul_rn(__dadd_rn(2.0, -rho), first),
                     -__dmul_rn(__dmul_rn(__dadd_rn(1.0, -rho), y), second));
      return isfinite(*g) && isfinite(*h) && *h > 0.0;
    }
    default:
      return false;
  }
}

// ComputeMulticlassSoftmaxGradients for one row (objective.cpp:130-152, 242-287): the
// class probability from the row's K margins (exp of each margin minus the maximum,
// normalized by their sum in class order), g = p - [label == target], h = p (1 - p).
__device__ __forceinline__ bool softmax_pair(const TrainerDev& a, double label, uint32_t row,
                                             uint32_t target, double* g, double* h) {
  const uint32_t K = a.n_classes;
  if (!f64_finite(label) || floor(label) != label || label < 0.0 || label >= double(K)) return false;
  double maximum = -INFINITY;
  for (uint32_t k = 0; k < K; ++k) {
    const double m = a.preds[size_t(k) * a.n_rows + row];
    if (!f64_finite(m)) return false;
    maximum = fmax(maximum, m);
  }
  double normalizer = 0.0, target_exp = 0.0;
  for (uint32_t k = 0; k < K; ++k) {
    const double e = exp(__dadd_rn(a.preds[size_t(k) * a.n_rows + row], -maximum));
    normalizer = __dadd_rn(normalizer, e);
    if (k == target) target_exp = e;
  }
  if (!f64_finite(normalizer) || normalizer <= 0.0) return false;
  const double p = __ddiv_rn(target_exp, normalizer);
  *g = __dadd_rn(p, uint32_t(label) == target ? -1.0 : 0.0);
  *h = __dmul_rn(p, __dadd_rn(1.0, -p));
  return f64_finite(*g) && f64_finite(*h) && *h >= 0.0;
}

// x / y for the split screen: the fast reciprocal division (within 2 ulp) where the
// divisor is a normal float below 2^125, the IEEE division elsewhere.
__device__ __forceinline__ float screen_div(float x, float y) {
  return (y > 0x1p-125f && y < 0x1p125f) ? __fdividef(x, y) : __fdiv_rn(x, y);
}

// True for a double with the sign bit set and a non-zero magnitude (x < 0).
__device__ __forceinline__ bool f64_negative(double x) {
  const long long b = __double_as_longlong(x);
  return b < 0 && (b & 0x7FFFFFFFFFFFFFFFll) != 0;
}

// grid = (x, n_trees): blockIdx.y is the tree, so a block's maxima belong to one tree.
// SQ: squared error without softmax classes only; the instantiation leaves out the other
// objectives' code, so it needs fewer registers and more rows are in flight per SM.
template <bool SQ>
__global__ void __launch_bounds__(256) gradients_kernel(TrainerDev a) {
  __shared__ uint32_t sg[8], shh[8];
  const uint32_t t = blockIdx.y;
  const size_t tree_off = size_t(t) * a.n_rows;
  // Squared error and quantile have h = 1, so h * w = w exactly.
  const bool unit_h = !a.n_classes && (a.objective == 0 || a.objective == 2);
  const long long class_bits = __double_as_longlong(double(t));
  uint32_t mg = 0, mh = 0, bad = 0;
  // Position p of the tree's root segment holds row i: the identity for boosting, the
  // tree's sample for a forest.
  const uint32_t count = a.sample_rows ? a.sample_count[t] : a.n_rows;
  const size_t pos_off = size_t(t) * 2 * a.seg_stride;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < count; p += gridDim.x * blockDim.x) {
    const uint32_t i = a.sample_rows ? a.sample_rows[size_t(t) * a.seg_stride + p] : p;
    if (i >= a.n_rows) {
      bad = 1;
      continue;
    }
    double y = a.labels[i];
    if (a.ovr) {  // y == t (class ids are non-negative integers; -0.0 equals class 0)
      const long long yb = __double_as_longlong(y);
      y = (yb == class_bits || (t == 0 && (yb << 1) == 0)) ? 1.0 : 0.0;
    }
    double g = 0.0, h = 0.0;
    if (SQ || (a.objective == 0 && !a.n_classes)) {
      // Squared error (the objective_pair case 0 then the weight products): g = w (p - y),
      // h = w; two FP64 operations per row on the narrow FP64 pipe.
      const double pred = a.preds[tree_off + i];
      g = __dsub_rn(pred, y);  // p + (-y): negation is exact
      if (!f64_finite(y) || !f64_finite(pred) || !f64_finite(g)) bad = 1;
      h = 1.0;
      if (a.weights != nullptr) {
        const double w = a.weights_per_tree ? a.weights[tree_off + i] : a.weights[i];
        g = __dmul_rn(g, w);
        h = w;
        if (!f64_finite(g) || !f64_finite(h) || f64_negative(h)) bad = 1;
      }
    } else if constexpr (!SQ) {
      if (a.n_classes) {
        if (!softmax_pair(a, y, i, *a.round_counter % a.n_classes, &g, &h)) bad = 1;
      } else {
        const double pred = a.preds[tree_off + i];
        if (!objective_pair(a.objective, y, pred, a.params, &g, &h)) bad = 1;
      }
      if (a.weights != nullptr) {
        const double w = a.weights_per_tree ? a.weights[tree_off + i] : a.weights[i];
        g = __dmul_rn(g, w);
        h = unit_h ? w : __dmul_rn(h, w);
        if (!f64_finite(g) || !f64_finite(h) || f64_negative(h)) bad = 1;
      }
    }
    const float g32 = f64_to_f32_rn(g), h32 = f64_to_f32_rn(h);
    if (!isfinite(g32) || !isfinite(h32)) bad = 1;
    a.gh[pos_off + p] = make_float2(g32, h32);  // parity 0 = the root segment's order
    a.rows[pos_off + p] = i;
    mg = max(mg, __float_as_uint(fabsf(g32)));
    mh = max(mh, __float_as_uint(fmaxf(h32, 0.0f)));
  }
  for (int off = 16; off > 0; off >>= 1) {
    mg = max(mg, __shfl_xor_sync(0xffffffffu, mg, off));
    mh = max(mh, __shfl_xor_sync(0xffffffffu, mh, off));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sg[warp] = mg;
    shh[warp] = mh;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < int(blockDim.x >> 5); ++w) {
      mg = max(mg, sg[w]);
      mh = max(mh, shh[w]);
    }
    atomicMax(&a.trees[t].max_abs_g_bits, mg);
    atomicMax(&a.trees[t].max_h_bits, mh);
  }
  if (bad) raise(a.ctl, kErrGradient);
}

__device__ __forceinline__ uint32_t root_rows(const TrainerDev& a, uint32_t t) {
  return a.sample_rows ? a.sample_count[t] : a.n_rows;
}

__global__ void round_setup_kernel(TrainerDev a) {
  if (threadIdx.x == 0) {  // trees are few: serial prefix of the roots' work items
    uint64_t total = 0;
    for (uint32_t t = 0; t < a.n_trees; ++t) total += root_rows(a, t);
    const uint32_t item_rows =
        a.item_rows ? a.item_rows : adaptive_item_rows(total, a.nfb, a.sm_count, a.items_per_sm);
    uint32_t acc = 0;
    for (uint32_t t = 0; t < a.n_trees; ++t) {
      a.build_prefix[t] = acc;
      acc += ceil_div(root_rows(a, t), item_rows);
    }
    a.build_prefix[a.n_trees] = acc;
    a.ctl->free_top = a.n_slots - a.n_trees;
    a.ctl->n_nodes = a.n_trees;
    a.ctl->n_build = a.n_trees;
    a.ctl->n_sub = 0;
    a.ctl->n_part = 0;
    a.ctl->hist_items = acc * a.nfb;
    a.ctl->hist_counter = 0;
    a.ctl->split_items = a.n_trees * a.n_fchunks;
    a.ctl->item_rows = item_rows;
  }
  for (uint32_t base = 0; base < a.n_trees; base += blockDim.x) {
    const uint32_t t = base + threadIdx.x;
    if (t < a.n_trees) {
      TreeState& s = a.trees[t];
      const float mg = __uint_as_float(s.max_abs_g_bits), mh = __uint_as_float(s.max_h_bits);
      // every row's |q| <= 2^30: the histogram's 32-bit limb sums cannot overflow
      s.kg = mg > 0.0f ? 30 - exponent_above(mg) : 0;
      s.kh = mh > 0.0f ? 30 - exponent_above(mh) : 0;
      s.inv_g = ldexp(1.0, -s.kg);
      s.inv_h = ldexp(1.0, -s.kh);
      const uint32_t slot = a.free_stack[a.n_slots - 1 - t];
      const uint32_t cnt = root_rows(a, t);
      NodeRec r;
      r.seg_off = 0;
      r.seg_cnt = cnt;
      r.node_index = 0;
      r.slot = slot;
      r.count = 0;
      r.qg = r.qh = 0;
      r.g = r.h = 0.0;
      r.lo = -INFINITY;
      r.hi = INFINITY;
      r.tree = t;
      r.depth = 0;
      r.sub_from = 0;
      a.nodes[0][t] = r;
      for (uint32_t w = 0; w < a.params.path_words; ++w) {
        uint32_t allowed = 0xffffffffu;
        if (a.params.n_groups > 0) {  // empty path: any group containing the feature
          allowed = 0;
          for (uint32_t g = 0; g < a.params.n_groups; ++g)
            allowed |= a.group_masks[g * a.params.path_words + w];
        }
        if (a.tree_feature_masks != nullptr)
          allowed &= a.tree_feature_masks[t * a.params.path_words + w];
        a.node_path[0][t * a.params.path_words + w] = 0;
        a.node_allowed[0][t * a.params.path_words + w] = allowed;
      }
      BuildEntry e;
      e.tree = t;
      e.parity = 0;
      e.seg_off = 0;
      e.seg_cnt = cnt;
      e.slot = slot;
      e.pad = 0;
      a.build[t] = e;
    }
  }
}

// Zero the histogram slots of the current build list.
__global__ void zero_build_slots_kernel(TrainerDev a) {
  // The level's split scan publishes node maxima into node_screen: clear them first.
  if (a.node_screen)
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.max_level_nodes; i += gridDim.x * blockDim.x)
      a.node_screen[i] = 0u;
  const uint64_t words_per_slot = uint64_t(a.features) * a.slots * 3;
  const uint64_t total = uint64_t(a.ctl->n_build) * (words_per_slot / 2);
  for (uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; idx < total;
       idx += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t e = uint32_t(idx / (words_per_slot / 2));
    const uint64_t w = idx % (words_per_slot / 2);
    if (a.tree_feature_masks) {
      // A forest tree reads only its own features' histograms (and feature 0's, for the
      // root statistics): the others are neither cleared nor subtracted nor scanned.
      const uint32_t f = uint32_t(w * 2 / (a.slots * 3));
      const uint32_t mask = a.tree_feature_masks[size_t(a.build[e].tree) * a.params.path_words + (f >> 5)];
      if (f != 0 && !((mask >> (f & 31)) & 1u)) continue;
    }
    reinterpret_cast<ulonglong2*>(a.hist + a.build[e].slot * words_per_slot)[w] =
        make_ulonglong2(0, 0);
  }
}

// The root of every tree holds all rows in every round, so its count histogram never
// changes, and when the hessian does not depend on the prediction (squared error and
// quantile: h = weight) neither does its hessian histogram, nor the hessian scale. The
// first round of a fit builds the roots in full and saves those two words per cell; later
// rounds build only the gradient limbs and restore them. The hessian scale is checked.
__global__ void root_cache_kernel(TrainerDev a, int save) {
  const uint64_t per_tree = uint64_t(a.features) * a.slots;
  const uint64_t total = per_tree * a.n_trees;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < total;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t t = uint32_t(i / per_tree);
    const uint64_t cell = i % per_tree;
    unsigned long long* slot = a.hist + (uint64_t(a.build[t].slot) * per_tree + cell) * 3;
    unsigned long long* c = a.root_cache + i * 2;
    if (save) {
      c[0] = slot[0];
      c[1] = slot[2];
      if (cell == 0) a.root_cache_kh[t] = a.trees[t].kh;
    } else {
      if (a.root_cache_kh[t] != a.trees[t].kh) {
        if (cell == 0) raise(a.ctl, kErrRootCache);
        continue;
      }
      slot[0] = c[0];
      slot[2] = c[1];
    }
  }
}

// Root statistics: the total of feature 0's slots (all rows, exact in fixed mode).
__global__ void root_stats_kernel(TrainerDev a) {
  const int lane = threadIdx.x & 31;
  for (uint32_t t = threadIdx.x >> 5; t < a.n_trees; t += blockDim.x >> 5) {
    NodeRec& r = a.nodes[0][t];
    const unsigned long long* base = a.hist + size_t(r.slot) * a.features * a.slots * 3;
    unsigned long long cnt = 0;
    long long qg = 0, qh = 0;
    for (uint32_t s = lane; s < a.slots; s += 32) {
      cnt += base[s * 3 + 0];
      qg += (long long)base[s * 3 + 1];
      qh += (long long)base[s * 3 + 2];
    }
    for (int off = 16; off > 0; off >>= 1) {
      cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
      qg += __shfl_xor_sync(0xffffffffu, qg, off);
      qh += __shfl_xor_sync(0xffffffffu, qh, off);
    }
    if (lane == 0) {
      const TreeState& st = a.trees[t];
      r.count = cnt;
      if (a.mode == kModeFixed) {
        r.qg = qg;
        r.qh = qh;
        r.g = q_image(qg, st.inv_g);
        r.h = q_image(qh, st.inv_h);
      } else {  // FP64 total in slot order
        double g = 0.0, h = 0.0;
        for (uint32_t s = 0; s < a.slots; ++s) {
          g = __dadd_rn(g, __longlong_as_double((long long)base[s * 3 + 1]));
          h = __dadd_rn(h, __longlong_as_double((long long)base[s * 3 + 2]));
        }
        r.g = g;
        r.h = h;
      }
      if (cnt != r.seg_cnt) raise(a.ctl, kErrCountMismatch);
      double leaf = 0.0;
      if (!leaf_weight(r.g, r.h, a.params, &leaf)) raise(a.ctl, kErrNonFinite);
      TreeNodeOut n;
      n.feature_index = 0;
      n.threshold_bin = 0;
      n.left_child = 0xffffffffu;
      n.right_child = 0xffffffffu;
      n.leaf_value = leaf;
      n.gain = 0.0;
      n.default_left = 1;
      n.flags = 1;
      for (int k = 0; k < 6; ++k) n.reserved[k] = 0;
      a.tree_nodes[size_t(t) * a.max_tree_nodes] = n;
    }
  }
}

// slot_parent := slot_parent - slot_built for every pair (the parent slot becomes the
// sibling's histogram).
__global__ void subtract_kernel(TrainerDev a) {
  const uint64_t bins_per_slot = uint64_t(a.features) * a.slots;
  const uint64_t total = uint64_t(a.ctl->n_sub) * bins_per_slot;
  uint32_t err = 0;
  for (uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; idx < total;
       idx += uint64_t(gridDim.x) * blockDim.x) {
    const SubEntry e = a.sub[idx / bins_per_slot];
    const uint64_t b = idx % bins_per_slot;
    if (a.tree_feature_masks) {  // a forest tree's own features only (sub[k] pairs build[k])
      const uint32_t f = uint32_t(b / a.slots);
      const uint32_t mask =
          a.tree_feature_masks[size_t(a.build[idx / bins_per_slot].tree) * a.params.path_words + (f >> 5)];
      if (!((mask >> (f & 31)) & 1u)) continue;
    }
    unsigned long long* p = a.hist + (e.parent_slot * bins_per_slot + b) * 3;
    const unsigned long long* c = a.hist + (e.built_slot * bins_per_slot + b) * 3;
    const unsigned long long pc = p[0], cc = c[0];
    if (cc > pc) err |= kErrSubtraction;
    p[0] = pc - cc;
    if (a.mode == kModeFixed) {
      p[1] = p[1] - c[1];
      p[2] = p[2] - c[2];
    } else {
      const double pg = __longlong_as_double((long long)p[1]);
      const double cg = __longlong_as_double((long long)c[1]);
      const double g = __dadd_rn(pg, -cg);
      if (!isfinite(pg) || !isfinite(cg) || !isfinite(g)) err |= kErrNonFinite;
      const double ph = __longlong_as_double((long long)p[2]);
      const double ch = __longlong_as_double((long long)c[2]);
      if (!isfinite(ph) || !isfinite(ch) || ph < 0.0 || ch < 0.0) err |= kErrHessian;
      const double diff = __dadd_rn(ph, -ch);
      const double tol = __dmul_rn(1e-5, fmax(1.0, fmax(fabs(ph), fabs(ch))));
      if (diff < -tol) err |= kErrSubtraction;
      p[1] = (unsigned long long)__double_as_longlong(g);
      p[2] = (unsigned long long)__double_as_longlong(diff < 0.0 ? 0.0 : diff);
    }
  }
  if (err) raise(a.ctl, err);
}

// ------------------------------------------------------------------------------------
// Split scan
// ------------------------------------------------------------------------------------
// Node statistics of the scan: exact int64 (fixed) or FP64 (float).
template <bool FIXED>
struct Stat {
  using V = typename std::conditional<FIXED, long long, double>::type;
  uint32_t count;  // a node holds fewer than 2^32 rows
  V g, h;
};

template <bool FIXED>
__device__ __forceinline__ Stat<FIXED> stat_zero() {
  Stat<FIXED> r;
  r.count = 0;
  r.g = 0;
  r.h = 0;
  return r;
}

template <bool FIXED>
__device__ __forceinline__ Stat<FIXED> stat_add(Stat<FIXED> x, Stat<FIXED> y) {
  Stat<FIXED> r;
  r.count = x.count + y.count;
  if constexpr (FIXED) {
    r.g = x.g + y.g;
    r.h = x.h + y.h;
  } else {
    r.g = __dadd_rn(x.g, y.g);
    r.h = __dadd_rn(x.h, y.h);
  }
  return r;
}

template <bool FIXED>
__device__ __forceinline__ Stat<FIXED> stat_sub(Stat<FIXED> x, Stat<FIXED> y) {
  Stat<FIXED> r;
  r.count = x.count - y.count;
  if constexpr (FIXED) {
    r.g = x.g - y.g;
    r.h = x.h - y.h;
  } else {
    r.g = __dadd_rn(x.g, -y.g);
    r.h = __dadd_rn(x.h, -y.h);
  }
  return r;
}

template <bool FIXED>
__device__ __forceinline__ Stat<FIXED> shfl_up_stat(Stat<FIXED> s, int off) {
  Stat<FIXED> r;
  r.count = __shfl_up_sync(0xffffffffu, s.count, off);
  r.g = __shfl_up_sync(0xffffffffu, s.g, off);
  r.h = __shfl_up_sync(0xffffffffu, s.h, off);
  return r;
}

template <bool FIXED>
__device__ __forceinline__ Stat<FIXED> shfl_stat(Stat<FIXED> s, int src) {
  Stat<FIXED> r;
  r.count = __shfl_sync(0xffffffffu, s.count, src);
  r.g = __shfl_sync(0xffffffffu, s.g, src);
  r.h = __shfl_sync(0xffffffffu, s.h, src);
  return r;
}

// q_image(x) > q_image(y), out of line: the FP64 conversions are not speculated into
// the common case.
static __device__ __noinline__ bool images_above(long long x, long long y, double inv) {
  return q_image(x, inv) > q_image(y, inv);
}

template <bool FIXED>
__device__ __forceinline__ double image(typename Stat<FIXED>::V v, double inv) {
  if constexpr (FIXED) return q_image(v, inv);
  else return v;
}

// ConsiderMissingDirection (tree_split.cpp:65-115) + MonotonicBoundsForSplit
// (tree_monotonic.cpp:12-58).
template <bool FIXED>
__device__ __forceinline__ void consider(const TreeParams& p, const Stat<FIXED>& cl,
                                         const Stat<FIXED>& cr, double inv_g, double inv_h,
                                         int8_t mono, double plo, double phi, uint32_t feature,
                                         uint32_t threshold, uint32_t default_left,
                                         SplitRec& best, uint32_t& err) {
  if (cl.count < p.min_samples_leaf || cr.count < p.min_samples_leaf) return;
  const double lh = image<FIXED>(cl.h, inv_h), rh = image<FIXED>(cr.h, inv_h);
  if (lh < p.min_child_weight || rh < p.min_child_weight || lh <= 0.0 || rh <= 0.0) return;
  const double lg = image<FIXED>(cl.g, inv_g), rg = image<FIXED>(cr.g, inv_g);
  double gain;
  if (!split_gain(lg, lh, rg, rh, p, &gain)) {
    err |= kErrNonFinite;
    return;
  }
  if (gain <= 0.0 || gain < p.min_gain_to_split) return;
  double ll = plo, lu = phi, rl = plo, ru = phi;
  if (mono != 0) {
    double lv, rv;
    if (!leaf_weight(lg, lh, p, &lv) || !leaf_weight(rg, rh, p, &rv)) {
      err |= kErrNonFinite;
      return;
    }
    lv = clamp_bounds(lv, plo, phi);
    rv = clamp_bounds(rv, plo, phi);
    if (mono > 0) {
      if (lv > rv) return;
      lu = (rv < lu) ? rv : lu;  // std::min(lu, rv)
      rl = (rl < lv) ? lv : rl;  // std::max(rl, lv)
    } else {
      if (lv < rv) return;
      ll = (ll < rv) ? rv : ll;  // std::max(ll, rv)
      ru = (lv < ru) ? lv : ru;  // std::min(ru, lv)
    }
  }
  SplitRec c;
  c.gain = gain;
  c.valid = 1;
  c.feature = feature;
  c.threshold = threshold;
  c.default_left = default_left;
  c.lcount = cl.count;
  c.rcount = cr.count;
  if constexpr (FIXED) {
    c.lqg = cl.g;
    c.lqh = cl.h;
    c.rqg = cr.g;
    c.rqh = cr.h;
  } else {
    c.lqg = c.lqh = c.rqg = c.rqh = 0;
  }
  c.lg = lg;
  c.lh = lh;
  c.rg = rg;
  c.rh = rh;
  c.ll = ll;
  c.lu = lu;
  c.rl = rl;
  c.ru = ru;
  if (better_split(c, best)) best = c;
}

// One warp per (node, feature); a CTA covers one node and blockDim/32 features and
// writes the best split of its features to partial[node][chunk].
constexpr int kScanThreadsMax = 512;
constexpr uint32_t kScanQueue = 32;  // FP64 candidates queued per warp

// A candidate waiting for the exact FP64 evaluation.
template <bool FIXED>
struct ScanCand {
  Stat<FIXED> cl, cr;
  uint32_t threshold, default_left;
};

// A feature's histogram staged in shared memory, [word][k][lane] for slot lane * 8 + k
// (word 0 count, 1 g, 2 h): the lane's eight slots read conflict-free.
constexpr size_t kScanHistBytes = size_t(kSlots) * 3 * sizeof(unsigned long long);

// Shared memory per warp: its best split, its staged histogram and (exact phase) its FP64
// queue.
template <bool FIXED, bool SCREEN>
constexpr size_t scan_smem_per_warp() {
  return sizeof(SplitRec) + kScanHistBytes + (SCREEN ? 0 : kScanQueue * sizeof(ScanCand<FIXED>));
}

// Copies a feature's histogram (kSlots x {count, g, h} 64-bit words, 6 KB, 16-byte
// aligned) into the warp's staging area with coalesced 16-byte loads, all in flight
// together.
__device__ __forceinline__ void stage_feature_hist(const unsigned long long* src,
                                                   unsigned long long* dst, int lane) {
  constexpr int kChunks = int(kScanHistBytes / 16);  // 384
  constexpr int kPerLane = kChunks / 32;              // 12
  constexpr int kBatch = 4;
  const ulonglong2* s2 = reinterpret_cast<const ulonglong2*>(src);
#pragma unroll 1
  for (int part = 0; part < kPerLane / kBatch; ++part) {
    ulonglong2 v[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) v[j] = __ldg(s2 + (part * kBatch + j) * 32 + lane);
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const uint32_t w0 = uint32_t((part * kBatch + j) * 32 + lane) * 2u;
#pragma unroll
      for (uint32_t q = 0; q < 2; ++q) {
        const uint32_t w = w0 + q, slot = w / 3u, word = w - slot * 3u;
        dst[(word * 8u + (slot & 7u)) * 32u + (slot >> 3)] = q ? v[j].y : v[j].x;
      }
    }
  }
  __syncwarp();
}

// stage_feature_hist of a sibling's histogram, formed on the way: parent minus the built
// child word by word, with subtract_kernel's checks (count underflow; float mode: finite
// sums, non-negative hessians, the hessian difference clamped at 0 within 1e-5), and
// written back over the parent's words in the same 16-byte chunks.
// One word of a sibling's slot: parent minus built child, with subtract_kernel's checks
// (word 0 count, 1 g, 2 h).
template <bool FIXED>
__device__ __forceinline__ unsigned long long sibling_word(unsigned long long pw, unsigned long long cw,
                                                           uint32_t word, uint32_t& err) {
  if (word == 0 || FIXED) {
    if (word == 0 && cw > pw) err |= kErrSubtraction;
    return pw - cw;
  }
  const double pd = __longlong_as_double((long long)pw), cd = __longlong_as_double((long long)cw);
  if (word == 1) {
    const double g = __dadd_rn(pd, -cd);
    if (!isfinite(pd) || !isfinite(cd) || !isfinite(g)) err |= kErrNonFinite;
    return (unsigned long long)__double_as_longlong(g);
  }
  if (!isfinite(pd) || !isfinite(cd) || pd < 0.0 || cd < 0.0) err |= kErrHessian;
  const double diff = __dadd_rn(pd, -cd);
  const double tol = __dmul_rn(1e-5, fmax(1.0, fmax(fabs(pd), fabs(cd))));
  if (diff < -tol) err |= kErrSubtraction;
  return (unsigned long long)__double_as_longlong(diff < 0.0 ? 0.0 : diff);
}

template <bool FIXED>
__device__ __forceinline__ void stage_sibling_hist(unsigned long long* parent,
                                                   const unsigned long long* built,
                                                   unsigned long long* dst, int lane, uint32_t& err) {
  constexpr int kChunks = int(kScanHistBytes / 16);  // 384
  constexpr int kPerLane = kChunks / 32;              // 12
  constexpr int kBatch = 4;
  ulonglong2* p2 = reinterpret_cast<ulonglong2*>(parent);
  const ulonglong2* c2 = reinterpret_cast<const ulonglong2*>(built);
#pragma unroll 1
  for (int part = 0; part < kPerLane / kBatch; ++part) {
    ulonglong2 pv[kBatch], cv[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      pv[j] = p2[(part * kBatch + j) * 32 + lane];
      cv[j] = c2[(part * kBatch + j) * 32 + lane];
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const uint32_t w0 = uint32_t((part * kBatch + j) * 32 + lane) * 2u;
      unsigned long long out[2];
#pragma unroll
      for (uint32_t q = 0; q < 2; ++q) {
        const unsigned long long pw = q ? pv[j].y : pv[j].x, cw = q ? cv[j].y : cv[j].x;
        const uint32_t w = w0 + q, word = w % 3u;
        const unsigned long long r = sibling_word<FIXED>(pw, cw, word, err);
        out[q] = r;
        const uint32_t slot = w / 3u;
        dst[(word * 8u + (slot & 7u)) * 32u + (slot >> 3)] = r;
      }
      p2[(part * kBatch + j) * 32 + lane] = make_ulonglong2(out[0], out[1]);
    }
  }
  __syncwarp();
}

// A feature with at most 32 bins: its slots 0-31 staged one per lane (slot l's words at
// dst[(w * 8) * 32 + l]) and its missing slot returned in *miss_words (every lane). All
// other slots are empty: every bin is below the feature's bin count. sub: parent minus the
// built child (`built`), written back as stage_sibling_hist does.
template <bool FIXED>
__device__ __forceinline__ void stage_few_slots(unsigned long long* slot_hist,
                                                const unsigned long long* built, bool hm,
                                                unsigned long long* dst, int lane,
                                                unsigned long long* miss_words, uint32_t& err) {
#pragma unroll
  for (uint32_t w = 0; w < 3; ++w) {
    const size_t at = size_t(lane) * 3 + w;
    unsigned long long v = slot_hist[at];
    if (built) {
      v = sibling_word<FIXED>(v, built[at], w, err);
      slot_hist[at] = v;
    }
    dst[(w * 8u) * 32u + uint32_t(lane)] = v;
  }
#pragma unroll
  for (uint32_t w = 0; w < 3; ++w) {
    const size_t at = size_t(kMissingSlot) * 3 + w;
    unsigned long long v = 0;
    if (hm) {
      v = slot_hist[at];
      if (built) {
        v = sibling_word<FIXED>(v, built[at], w, err);
        __syncwarp();
        if (lane == 0) slot_hist[at] = v;
      }
    }
    miss_words[w] = v;
  }
  __syncwarp();
}

// Bit 31 of a chunk's screen word: some feature of the chunk is evaluated exactly whatever
// the node's maximum (its screen is off, or a candidate is too close to call in FP32).
// The low bits hold the chunk's best certainly admissible FP32 score (a non-negative
// float's bits).
constexpr uint32_t kChunkExact = 0x80000000u;

// The split scan of a level, one warp per (node, feature), a CTA per (node, chunk of
// blockDim/32 features). With the FP32 screen on (best-split strategy, no reg_alpha,
// reg_lambda > 0) it runs in two launches:
//  SCREEN: each warp forms its feature's prefix sums and the FP32 scores of its
//    candidates, raises the node's running maximum of certainly admissible scores
//    (node_screen, atomicMax on the float bits) and writes its chunk's maximum and exact
//    flag (chunk_screen).
//  EXACT: with the node's final maximum M, a chunk whose candidates all score below
//    M(1 - 2^-18) and holds nothing to evaluate exactly writes "no split" at once; the
//    other chunks evaluate in FP64, as the reference does, every candidate at or above
//    that cut and every close call. A candidate below the cut has a strictly lower exact
//    gain than the admissible candidate that scored M, which its own chunk evaluates, so
//    it can win neither its chunk nor the node.
// EXACT alone (screen off, or no node maxima: the per-feature entry point) screens each
// feature against its own maximum. Each chunk's best split goes to partial[node][chunk].
//
// WIDE (a dataset with more than kSlots slots per feature): each warp walks its feature's
// slots in pages of kSlots, first for the total count and the missing slot (the last
// page's slot kMissingSlot), then per scan pass page by page with the left prefix carried
// from page to page; thresholds are numbered across pages.
template <bool FIXED, bool SCREEN, bool WIDE>
__global__ void __launch_bounds__(kScanThreadsMax) split_scan_kernel(TrainerDev a, int parity) {
  using V = typename Stat<FIXED>::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  SplitRec* warp_best = reinterpret_cast<SplitRec*>(smem_raw);
  uint32_t* warp_screen = reinterpret_cast<uint32_t*>(smem_raw);  // SCREEN: [warp]
  unsigned long long* s_hist =
      reinterpret_cast<unsigned long long*>(smem_raw + sizeof(SplitRec) * nwarps);
  ScanCand<FIXED>* s_queue = reinterpret_cast<ScanCand<FIXED>*>(
      smem_raw + (sizeof(SplitRec) + kScanHistBytes) * nwarps);
  static_assert(sizeof(SplitRec) % 8 == 0, "staged words and queue entries stay 8-byte aligned");
  __shared__ uint32_t s_list[32], s_listed;  // two-phase exact launch: a batch's items to evaluate
  const TreeParams& P = a.params;
  const uint32_t n_chunks = a.n_fchunks;
  const uint32_t n_nodes = a.ctl->n_nodes;
  const uint32_t items = n_nodes * n_chunks;
  const bool two_phase = !SCREEN && a.node_screen != nullptr && a.scan_two_phase != 0;
  // The level's first launch forms the siblings' histograms (u8 datasets).
  const bool fuse_sub = !WIDE && a.fused_sub != 0 && (SCREEN || !two_phase);
  // Launch-wide screen constants (FP64 tests and conversions stay out of the item loop).
  const bool screen_params = P.screen_params != 0;
  const float lam32 = P.screen_lambda;
  const bool mcw_on = P.screen_mcw_on != 0;
  const float mcw_lo = P.screen_mcw_lo, mcw_hi = P.screen_mcw_hi;
  // The work on one (node, chunk) item; every thread of the CTA calls it.
  auto eval_item = [&](uint32_t item) {
    const uint32_t i = item / n_chunks, c = item % n_chunks;
    const NodeRec node = a.nodes[parity][i];
    const uint32_t f = c * uint32_t(nwarps) + uint32_t(warp);
    const double inv_g = a.trees[node.tree].inv_g, inv_h = a.trees[node.tree].inv_h;
    const int st_kg = a.trees[node.tree].kg, st_kh = a.trees[node.tree].kh;
    SplitRec best;
    best.valid = 0;
    best.gain = 0.0;
    best.feature = f;
    best.threshold = 0;
    best.default_left = 1;
    uint32_t err = 0;
    float best32 = -1.0f;  // SCREEN: best certainly admissible FP32 score of the feature
    bool exact = false;    // SCREEN: the feature needs the exact pass whatever the cut
    // A node with fewer than 2 * min_samples_leaf rows has no admissible split.
    bool active = f < a.features && node.count >= 2 * P.min_samples_leaf;
    if (active) {
      const uint32_t allowed = a.node_allowed[parity][i * P.path_words + (f >> 5)];
      active = (allowed >> (f & 31)) & 1u;
    }
    if (active) {  // warp-uniform
      const uint32_t nb = a.bin_count[f];
      const bool hm = a.has_missing[f] != 0;
      // At most 32 bins: one slot per lane (slot = lane), the missing slot apart.
      const bool few = !WIDE && nb <= 32u;
      const int kper = few ? 1 : 8;
      unsigned long long* sh = s_hist + size_t(warp) * (kScanHistBytes / 8);
      const uint32_t pages = WIDE ? a.slots / uint32_t(kSlots) : 1u;
      const unsigned long long* fhist =
          a.hist + (size_t(node.slot) * a.features + f) * size_t(WIDE ? a.slots : uint32_t(kSlots)) * 3;
      // Slot lane * 8 + k of the staged page (few bins: slot lane, k = 0): word w at
      // sh[(w * 8 + k) * 32 + lane].
      auto slot_word = [&](int k, int w) -> unsigned long long { return sh[(w * 8 + k) * 32 + lane]; };
      auto slot_of = [&](int k) -> int { return few ? lane : lane * 8 + k; };
      // The lane's total of its 8 slots of the staged page; the missing slot (slot
      // kMissingSlot of the last page) goes to `miss` instead. Raw counts add to `count`.
      auto page_sums = [&](bool last, Stat<FIXED>& sum, Stat<FIXED>& miss,
                           unsigned long long& count) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (k >= kper) break;
          const int s = slot_of(k);
          Stat<FIXED> b;
          const unsigned long long raw_count = slot_word(k, 0);
          b.count = uint32_t(raw_count);  // the total below checks the full word
          if constexpr (FIXED) {
            b.g = (long long)slot_word(k, 1);
            b.h = (long long)slot_word(k, 2);
          } else {
            b.g = __longlong_as_double((long long)slot_word(k, 1));
            b.h = __longlong_as_double((long long)slot_word(k, 2));
            if (!isfinite(b.g) || !isfinite(b.h) || b.h < 0.0) err |= kErrNonFinite;
          }
          count += raw_count;
          if (hm && last && s == kMissingSlot) {
            miss = b;
          } else {
            sum = stat_add<FIXED>(sum, b);
          }
        }
      };
      auto inclusive_prefix = [&](Stat<FIXED> incl) -> Stat<FIXED> {
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const Stat<FIXED> y = shfl_up_stat<FIXED>(incl, off);
          if (lane >= off) incl = stat_add<FIXED>(y, incl);
        }
        return incl;
      };
      auto exclusive_of = [&](const Stat<FIXED>& incl) -> Stat<FIXED> {
        Stat<FIXED> cin = shfl_up_stat<FIXED>(incl, 1);
        if (lane == 0) cin = stat_zero<FIXED>();
        return cin;
      };
      Stat<FIXED> miss = stat_zero<FIXED>(), carry_in = stat_zero<FIXED>();
      unsigned long long total_count = 0;
      if constexpr (WIDE) {
        for (uint32_t p = 0; p < pages; ++p) {
          __syncwarp();
          stage_feature_hist(fhist + size_t(p) * kSlots * 3, sh, lane);
          Stat<FIXED> unused = stat_zero<FIXED>();
          page_sums(p + 1 == pages, unused, miss, total_count);
        }
      } else {
        const bool sub = fuse_sub && node.sub_from != 0;
        unsigned long long* own = a.hist + (size_t(node.slot) * a.features + f) * kSlots * 3;
        const unsigned long long* built =
            sub ? a.hist + (size_t(node.sub_from - 1) * a.features + f) * kSlots * 3 : nullptr;
        unsigned long long mw[3] = {0ull, 0ull, 0ull};
        if (few) {
          stage_few_slots<FIXED>(own, built, hm, sh, lane, mw, err);
        } else if (sub) {
          stage_sibling_hist<FIXED>(own, built, sh, lane, err);
        } else {
          stage_feature_hist(fhist, sh, lane);
        }
        Stat<FIXED> sum = stat_zero<FIXED>();
        page_sums(true, sum, miss, total_count);
        carry_in = exclusive_of(inclusive_prefix(sum));
        if (few) {  // the missing slot, in every lane; its rows counted once
          miss.count = uint32_t(mw[0]);
          if constexpr (FIXED) {
            miss.g = (long long)mw[1];
            miss.h = (long long)mw[2];
          } else {
            miss.g = __longlong_as_double((long long)mw[1]);
            miss.h = __longlong_as_double((long long)mw[2]);
            if (!isfinite(miss.g) || !isfinite(miss.h) || miss.h < 0.0) err |= kErrNonFinite;
          }
          if (lane == 0) total_count += mw[0];
        }
      }
      if (!few) miss = shfl_stat<FIXED>(miss, 31);
      for (int off = 16; off > 0; off >>= 1)
        total_count += __shfl_xor_sync(0xffffffffu, total_count, off);
      if (total_count != node.count) err |= kErrCountMismatch;
      Stat<FIXED> parent;
      parent.count = node.count;
      if constexpr (FIXED) {
        parent.g = node.qg;
        parent.h = node.qh;
      } else {
        parent.g = node.g;
        parent.h = node.h;
      }
      if (nb >= 2 && total_count == node.count) {
        bool miss_h_above;
        if constexpr (FIXED) {
          // The images q * 2^-k compare as the quantized sums while those convert exactly.
          const long long lim = 1ll << 53;
          miss_h_above = (miss.h > -lim && miss.h < lim && parent.h > -lim && parent.h < lim)
                             ? miss.h > parent.h
                             : images_above(miss.h, parent.h, inv_h);
        } else {
          miss_h_above = miss.h > parent.h;
        }
        if (miss.count > parent.count || miss_h_above) err |= kErrMissing;
        const Stat<FIXED> nmp = stat_sub<FIXED>(parent, miss);
        const int8_t mono = P.has_monotonic ? a.monotonic[f] : 0;
        const uint32_t rnd =
            P.split_strategy == 1
                ? stable_random_threshold(
                      a.tree_seeds ? a.tree_seeds[node.tree] : P.random_seed,
                      a.feature_rank ? a.feature_rank[size_t(node.tree) * a.features + f] : f,
                      node.node_index, node.depth, nb - 1)
                : 0xffffffffu;
        // Exact FP32 pre-screen. Every eligible candidate's score S = gL^2/(hL+lambda) +
        // gR^2/(hR+lambda) is computed in FP32 with relative error <= 14u (u = 2^-24; each
        // int64 -> FP32 conversion below is within 3u, lambda is rounded once, a division
        // within 2u). A candidate whose FP32 score is below M(1 - 2^-18), M the best FP32
        // score of a certainly eligible candidate of the node, then has an exact score at
        // least 30u*M below that candidate's, far outside the FP64 evaluation's own
        // rounding (a few 2^-53 * M, the parent score included), so its FP64 gain is
        // strictly lower and it cannot win. Only the rest -- and candidates whose
        // min_child_weight test or score is too close to call in FP32 -- run the FP64
        // evaluation of the reference. The score is quadratic only without reg_alpha, the
        // admissible set monotone in it only without monotone constraints, and random
        // thresholds leave one candidate: the screen is off for those, and where 2^-k
        // leaves the FP32 normal range.
        const bool screen = screen_params && mono == 0 &&
                            (!FIXED || (st_kg >= -120 && st_kg <= 120 && st_kh >= -120 && st_kh <= 120));
        // 2^-k exactly, built from the exponent field.
        const float inv_g32 = FIXED && screen ? __int_as_float((127 - st_kg) << 23) : 1.0f;
        const float inv_h32 = FIXED && screen ? __int_as_float((127 - st_kh) << 23) : 1.0f;
        // |v| as hi * 2^32 + lo: float(hi) and float(lo) are each within u, and the fused
        // multiply-add rounds once more, so the result is within 3u of v (no cancellation:
        // both parts are non-negative). The conversions run on the FP32 pipe.
        auto to32 = [&](V v, float inv32) -> float {
          if constexpr (FIXED) {
            const unsigned long long m = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
            const float f = __fmaf_rn(u32_to_f32_rn(uint32_t(m >> 32)), 4294967296.0f,
                                      u32_to_f32_rn(uint32_t(m)));
            return (v < 0 ? -f : f) * inv32;
          } else {
            return f64_to_f32_rn(v);
          }
        };
        // 0: rejected by the FP64 test before any arithmetic (no error flag either);
        // 1: admissible, FP32 score in *s32; 2: too close to call.
        auto classify = [&](const Stat<FIXED>& cl, const Stat<FIXED>& cr, float* s32) -> int {
          if (cl.count < P.min_samples_leaf || cr.count < P.min_samples_leaf) return 0;
          if constexpr (!FIXED) {
            if (!f64_finite(cl.h) || !f64_finite(cr.h) || !f64_finite(cl.g) || !f64_finite(cr.g)) return 2;
          }
          if (!(cl.h > 0) || !(cr.h > 0)) return 0;  // fixed point: image > 0 iff q > 0
          const float lh = to32(cl.h, inv_h32), rh = to32(cr.h, inv_h32);
          int cls = 1;
          if (mcw_on) {
            if (lh < mcw_lo || rh < mcw_lo) return 0;
            if (lh <= mcw_hi || rh <= mcw_hi) cls = 2;
          }
          const float lg = to32(cl.g, inv_g32), rg = to32(cr.g, inv_g32);
          const float sc = screen_div(lg * lg, lh + lam32) + screen_div(rg * rg, rh + lam32);
          if (!isfinite(sc)) cls = 2;
          *s32 = sc;
          return cls;
        };
        // Visits every (threshold, missing direction) step of the lane's 8 slots of the
        // staged page (the left prefix before them `cin`, the page's first threshold
        // `base`) with the candidate's left/right statistics; `cand` is false where no
        // candidate exists. Every lane visits every step (the visitor may use warp
        // collectives).
        auto scan_candidates = [&](const Stat<FIXED>& cin, uint32_t base, bool last, auto&& visit) {
          Stat<FIXED> left = cin;
#pragma unroll 1
          for (int k = 0; k < kper; ++k) {
            const int s = slot_of(k);
            bool empty_bin = false;
            if (!(hm && last && s == kMissingSlot)) {  // reload the slot from the staging area
              Stat<FIXED> b;
              b.count = uint32_t(slot_word(k, 0));
              empty_bin = b.count == 0;
              if constexpr (FIXED) {
                b.g = (long long)slot_word(k, 1);
                b.h = (long long)slot_word(k, 2);
              } else {
                b.g = __longlong_as_double((long long)slot_word(k, 1));
                b.h = __longlong_as_double((long long)slot_word(k, 2));
              }
              left = stat_add<FIXED>(left, b);
            }
            const uint32_t t = base + uint32_t(s);
            const Stat<FIXED> right = stat_sub<FIXED>(nmp, left);
            bool cand = t + 1 < nb;
            if (cand && left.count > nmp.count) {
              err |= kErrPrefix;
              cand = false;
            }
            if (left.count == 0 && right.count == 0) cand = false;
            if (P.split_strategy == 1 && t != rnd) cand = false;
            // After an empty bin the candidate repeats threshold t-1's statistics exactly
            // and loses the tie to it (IsBetterSplit prefers the lower threshold).
            if (P.split_strategy == 0 && t > 0 && empty_bin) cand = false;
            for (int d = 0; d < 2; ++d) {
              const uint32_t dl = 1u - uint32_t(d);  // default_left 1, then 0
              if (dl == 0 && miss.count == 0) break;  // warp-uniform
              const Stat<FIXED> cl = dl ? stat_add<FIXED>(left, miss) : left;
              const Stat<FIXED> cr = dl ? right : stat_add<FIXED>(right, miss);
              visit(cand, cl, cr, t, dl);
            }
          }
        };
        // Runs body(left prefix, first threshold, last page) for each page: the one page
        // staged above, or (wide) each page staged in turn with the prefix carried over.
        auto for_pages = [&](auto&& body) {
          if constexpr (!WIDE) {
            body(carry_in, 0u, true);
          } else {
            Stat<FIXED> carry = stat_zero<FIXED>();
            for (uint32_t p = 0; p < pages; ++p) {
              __syncwarp();
              stage_feature_hist(fhist + size_t(p) * kSlots * 3, sh, lane);
              const bool last = p + 1 == pages;
              Stat<FIXED> sum = stat_zero<FIXED>(), unused = stat_zero<FIXED>();
              unsigned long long unused_count = 0;
              page_sums(last, sum, unused, unused_count);
              const Stat<FIXED> incl = inclusive_prefix(sum);
              body(stat_add<FIXED>(carry, exclusive_of(incl)), p * uint32_t(kSlots), last);
              carry = stat_add<FIXED>(carry, shfl_stat<FIXED>(incl, 31));
            }
          }
        };
        // The lane's best certainly admissible FP32 score; close calls set `exact`.
        auto screen_scores = [&]() {
          for_pages([&](const Stat<FIXED>& cin, uint32_t base, bool last) {
            scan_candidates(cin, base, last, [&](bool cand, const Stat<FIXED>& cl,
                                                 const Stat<FIXED>& cr, uint32_t, uint32_t) {
              if (!cand) return;
              float sc = 0.0f;
              const int cls = classify(cl, cr, &sc);
              if (cls == 1) best32 = fmaxf(best32, sc);
              if (cls == 2) exact = true;
            });
          });
          for (int off = 16; off > 0; off >>= 1)
            best32 = fmaxf(best32, __shfl_xor_sync(0xffffffffu, best32, off));
        };
        if constexpr (SCREEN) {
          if (screen) screen_scores();
          else exact = true;
        } else {
          float cut = -1.0f;
          if (screen) {
            float m;
            if (two_phase) {
              m = __uint_as_float(a.node_screen[i]);
            } else {
              screen_scores();
              m = best32;
            }
            cut = m >= 1e-30f ? m * (1.0f - 0x1p-18f) : -1.0f;
          }
          // Candidates that pass the screen queue up, and the warp evaluates them in FP64
          // one per lane: the narrow FP64 pipe runs one pass per 32 survivors instead of
          // one per (threshold, direction) step that has a survivor in any lane.
          ScanCand<FIXED>* queue = s_queue + size_t(warp) * kScanQueue;
          uint32_t queued = 0;
          auto drain = [&]() {
            __syncwarp();
            if (uint32_t(lane) < queued) {
              const ScanCand<FIXED> e = queue[lane];
              consider<FIXED>(P, e.cl, e.cr, inv_g, inv_h, mono, node.lo, node.hi, f, e.threshold,
                              e.default_left, best, err);
            }
            __syncwarp();
            queued = 0;
          };
          for_pages([&](const Stat<FIXED>& cin, uint32_t base, bool last) {
            scan_candidates(cin, base, last, [&](bool cand, const Stat<FIXED>& cl,
                                                 const Stat<FIXED>& cr, uint32_t t, uint32_t dl) {
              bool want = cand;
              if (want && screen && cut > 0.0f) {
                float sc = 0.0f;
                const int cls = classify(cl, cr, &sc);
                want = cls == 2 || (cls == 1 && sc >= cut);
              }
              const uint32_t ballot = __ballot_sync(0xffffffffu, want);
              if (ballot == 0) return;
              const uint32_t n_new = uint32_t(__popc(ballot));
              if (queued + n_new > kScanQueue) drain();
              if (want) {
                ScanCand<FIXED> e;
                e.cl = cl;
                e.cr = cr;
                e.threshold = t;
                e.default_left = dl;
                queue[queued + uint32_t(__popc(ballot & ((1u << lane) - 1u)))] = e;
              }
              queued += n_new;
            });
          });
          if (queued) drain();
        }
      }
    }
    if (err) raise(a.ctl, err);
    if constexpr (SCREEN) {
      exact = __any_sync(0xffffffffu, exact);
      if (lane == 0) {
        if (best32 >= 1e-30f) atomicMax(a.node_screen + i, __float_as_uint(best32));
        warp_screen[warp] = (exact ? kChunkExact : 0u) | (best32 > 0.0f ? __float_as_uint(best32) : 0u);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t word = 0;
        for (int w = 0; w < nwarps; ++w)
          word = (word & kChunkExact) | (warp_screen[w] & kChunkExact) |
                 max(word & ~kChunkExact, warp_screen[w] & ~kChunkExact);
        a.chunk_screen[size_t(i) * n_chunks + c] = word;
      }
      __syncthreads();
    } else {
      // Warp argmax (all lanes share the feature): every lane ends with the winner's id.
      uint32_t win = uint32_t(lane);
      {
        double g = best.gain;
        uint32_t v = best.valid, thr = best.threshold, dl = best.default_left;
        for (int off = 16; off > 0; off >>= 1) {
          const double og = __shfl_xor_sync(0xffffffffu, g, off);
          const uint32_t ov = __shfl_xor_sync(0xffffffffu, v, off);
          const uint32_t ot = __shfl_xor_sync(0xffffffffu, thr, off);
          const uint32_t od = __shfl_xor_sync(0xffffffffu, dl, off);
          const uint32_t ow = __shfl_xor_sync(0xffffffffu, win, off);
          bool take;
          if (ov != v) take = ov > v;
          else if (!v) take = ow < win;
          else if (og != g) take = og > g;
          else if (ot != thr) take = ot < thr;
          else if (od != dl) take = od > dl;
          else take = ow < win;
          if (take) {
            g = og;
            v = ov;
            thr = ot;
            dl = od;
            win = ow;
          }
        }
      }
      if (uint32_t(lane) == win) warp_best[warp] = best;
      __syncthreads();
      if (threadIdx.x == 0) {
        SplitRec b = warp_best[0];
        for (int w = 1; w < nwarps; ++w)
          if (better_split(warp_best[w], b)) b = warp_best[w];
        a.partial[size_t(i) * n_chunks + c] = b;
      }
      __syncthreads();
    }
  };
  if (two_phase) {
    // Batches of 32 consecutive items: warp 0 tests them against their nodes' final screen
    // maxima, one lane each, writes "no split" for the chunks below the cut and lists the
    // rest, which the CTA then evaluates in turn. At the deep levels most chunks are below
    // the cut, and a CTA that tested them one at a time waited on a global load and two
    // barriers per chunk.
    const uint32_t n_batches = (items + 31u) / 32u;
    for (uint32_t bt = blockIdx.x; bt < n_batches; bt += gridDim.x) {
      if (warp == 0) {
        const uint32_t item = bt * 32u + uint32_t(lane);
        bool keep = false;
        if (item < items) {
          const uint32_t i = item / n_chunks, c = item % n_chunks;
          const uint32_t cs = a.chunk_screen[size_t(i) * n_chunks + c];
          const float m = __uint_as_float(a.node_screen[i]);
          keep = (cs & kChunkExact) || !(m >= 1e-30f) || !(__uint_as_float(cs) < m * (1.0f - 0x1p-18f));
          if (!keep) {
            SplitRec none;
            none.valid = 0;
            none.gain = 0.0;
            none.feature = c * uint32_t(nwarps);
            none.threshold = 0;
            none.default_left = 1;
            a.partial[size_t(i) * n_chunks + c] = none;
          }
        }
        const uint32_t ballot = __ballot_sync(0xffffffffu, keep);
        if (keep) s_list[__popc(ballot & ((1u << lane) - 1u))] = item;
        if (lane == 0) s_listed = uint32_t(__popc(ballot));
      }
      __syncthreads();
      const uint32_t listed = s_listed;
      for (uint32_t k = 0; k < listed; ++k) eval_item(s_list[k]);
      __syncthreads();  // the list is rewritten by the next batch
    }
  } else {
    for (uint32_t item = blockIdx.x; item < items; item += gridDim.x) eval_item(item);
  }
  (void)sizeof(V);
}

// ------------------------------------------------------------------------------------
// Level finalize (one CTA)
// ------------------------------------------------------------------------------------
__device__ void write_leaf(TreeNodeOut* dst, double value) {
  TreeNodeOut n;
  n.feature_index = 0;
  n.threshold_bin = 0;
  n.left_child = 0xffffffffu;
  n.right_child = 0xffffffffu;
  n.leaf_value = value;
  n.gain = 0.0;
  n.default_left = 1;
  n.flags = 1;
  for (int k = 0; k < 6; ++k) n.reserved[k] = 0;
  *dst = n;
}

__device__ bool bounded_leaf(const TreeParams& p, double g, double h, double lo, double hi,
                             double* out) {
  if (lo > hi) return false;
  double w;
  if (!leaf_weight(g, h, p, &w)) return false;
  *out = clamp_bounds(w, lo, hi);
  return true;
}

__global__ void __launch_bounds__(1024) finalize_kernel(TrainerDev a, int parity, uint32_t depth) {
  __shared__ uint32_t sh[33 * 6];
  Control* ctl = a.ctl;
  const TreeParams& P = a.params;
  const uint32_t n = ctl->n_nodes;
  const uint32_t W = P.path_words;
  const bool last = depth + 1 >= P.max_depth;  // children are leaves
  const uint32_t* tree_base = a.tree_scratch;                 // [T] valid prefix at first node
  uint32_t* tree_acc_base = a.tree_scratch + a.n_trees;       // [T] accepted prefix at first node
  uint32_t* tree_acc = a.tree_scratch + 2 * a.n_trees;        // [T] accepted count
  uint32_t* tree_vbase = a.tree_scratch;
  for (uint32_t t = threadIdx.x; t < a.n_trees; t += blockDim.x) tree_acc[t] = 0;
  __syncthreads();

  // Phase A0: one warp per node merges the best splits of the node's feature chunks into
  // chunk 0's record (lanes read chunks in parallel; the features of different chunks
  // differ, so the total order of better_split has a unique winner among valid records).
  if (depth < P.max_depth) {  // nodes at max_depth never split (tree.cpp:152-154)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t nfc = a.n_fchunks;
    for (uint32_t i = warp; i < n; i += nw) {
      SplitRec* rec = a.partial + size_t(i) * nfc;
      uint32_t mine = lane < int(nfc) ? uint32_t(lane) : 0u;
      for (uint32_t c = lane + 32; c < nfc; c += 32)
        if (better_split(rec[c], rec[mine])) mine = c;
      uint32_t v = rec[mine].valid, f = rec[mine].feature, thr = rec[mine].threshold;
      uint32_t dl = rec[mine].default_left;
      double g = rec[mine].gain;
      for (int off = 16; off > 0; off >>= 1) {
        const uint32_t ov = __shfl_xor_sync(0xffffffffu, v, off);
        const double og = __shfl_xor_sync(0xffffffffu, g, off);
        const uint32_t of = __shfl_xor_sync(0xffffffffu, f, off);
        const uint32_t ot = __shfl_xor_sync(0xffffffffu, thr, off);
        const uint32_t od = __shfl_xor_sync(0xffffffffu, dl, off);
        const uint32_t om = __shfl_xor_sync(0xffffffffu, mine, off);
        bool take;
        if (ov != v) take = ov > v;
        else if (!v) take = om < mine;  // all invalid: keep chunk 0's record
        else if (og != g) take = og > g;
        else if (of != f) take = of < f;
        else if (ot != thr) take = ot < thr;
        else if (od != dl) take = od > dl;
        else take = om < mine;
        if (take) {
          v = ov;
          g = og;
          f = of;
          thr = ot;
          dl = od;
          mine = om;
        }
      }
      if (mine != 0) {  // copy the winner's record into chunk 0, word by word
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(rec + mine);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(rec);
        const unsigned long long w = lane < int(sizeof(SplitRec) / 8) ? src[lane] : 0ull;
        __syncwarp();
        if (lane < int(sizeof(SplitRec) / 8)) dst[lane] = w;
      }
    }
  }
  __syncthreads();

  // Phase A: valid flags, valid prefix; rows the next level builds.
  uint32_t carry = 0, built_units = 0;
  for (uint32_t base = 0; base < n; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    uint32_t v[2] = {0, 0};
    uint32_t tree = 0;
    bool first = false;
    if (i < n) {
      if (depth < P.max_depth) {
        const SplitRec& b = a.partial[size_t(i) * a.n_fchunks];
        v[0] = b.valid;
        if (b.valid) v[1] = uint32_t(((b.lcount <= b.rcount ? b.lcount : b.rcount) + 255) / 256);
      }
      tree = a.nodes[parity][i].tree;
      first = i == 0 || a.nodes[parity][i - 1].tree != tree;
    }
    uint32_t tot[2];
    const uint32_t own = v[0];
    block_scan<2>(v, tot, sh);
    if (i < n) {
      a.scratch_flags[i] = own;
      a.scratch_prefix[i] = carry + v[0];
      if (first) tree_vbase[tree] = carry + v[0];
    }
    carry += tot[0];
    built_units += tot[1];
    __syncthreads();
  }
  __syncthreads();
  // Work items per SM of the next level: a level of few large nodes loses more to each
  // item's fixed cost (zero, flush) than to load imbalance, a level of many nodes (each
  // with a partial last chunk) the other way round: one item fewer below 8 nodes here,
  // one more from 8 (measured on the 10M x 128 workload: 2 best for depths 1-3, 4 for
  // depths 4-7).
  const uint32_t base_per_sm = a.items_per_sm ? a.items_per_sm : 3u;
  const uint32_t level_per_sm = n >= 8 ? base_per_sm + 1 : (base_per_sm > 2 ? base_per_sm - 1 : base_per_sm);
  const uint32_t item_rows =
      a.item_rows ? a.item_rows : adaptive_item_rows(uint64_t(built_units) * 256, a.nfb, a.sm_count, level_per_sm);

  // Phase B1: acceptance under max_leaves, accepted prefix, chunk prefixes.
  // Scanned values: 0 accepted, 1 build chunks, 2 partition chunks, 3 leaf segments,
  // 4 leaf chunks, 5 freed slots.
  uint32_t carry6[6] = {0, 0, 0, 0, 0, 0};
  const uint32_t leafseg_base = ctl->n_leafseg;
  const uint32_t leafchunk_base = ctl->leaf_chunks;
  for (uint32_t base = 0; base < n; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    uint32_t v[6] = {0, 0, 0, 0, 0, 0};
    uint32_t tree = 0;
    bool first = false;
    if (i < n) {
      const NodeRec node = a.nodes[parity][i];
      tree = node.tree;
      first = i == 0 || a.nodes[parity][i - 1].tree != tree;
      const uint32_t within = a.scratch_prefix[i] - tree_base[tree];
      const bool acc = a.scratch_flags[i] && (a.trees[tree].leaf_count + within < P.max_leaves);
      v[0] = acc;
      if (acc) {
        const SplitRec& b = a.partial[size_t(i) * a.n_fchunks];
        const uint32_t built = uint32_t(b.lcount <= b.rcount ? b.lcount : b.rcount);
        if (!last) {
          v[1] = ceil_div(built, item_rows);
          v[2] = ceil_div(node.seg_cnt, kPartChunk);
        }
      }
      const bool leafseg = !acc || last;
      v[3] = leafseg;
      v[4] = leafseg ? ceil_div(node.seg_cnt, kApplyChunk) : 0;
      v[5] = (!acc && !last) ? 1u : 0u;
    }
    const uint32_t own0 = v[0];
    uint32_t tot[6];
    block_scan<6>(v, tot, sh);
    if (i < n) {
      a.scratch_flags[i] = own0;
      a.scratch_prefix[i] = carry6[0] + v[0];
      a.scratch_aux[i] = carry6[5] + v[5];
      if (first) tree_acc_base[tree] = carry6[0] + v[0];
      if (own0) {
        const uint32_t k = carry6[0] + v[0];
        if (!last) {
          a.build_prefix[k] = carry6[1] + v[1];
          a.part_prefix[k] = carry6[2] + v[2];
        }
      }
      if (!own0 || last) a.leaf_prefix[leafseg_base + carry6[3] + v[3]] = leafchunk_base + carry6[4] + v[4];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) carry6[k] += tot[k];
    __syncthreads();
  }
  const uint32_t n_acc = carry6[0];
  const uint32_t free_top = ctl->free_top;
  __syncthreads();

  // Phase B2: apply splits, next-level nodes, build / subtract / partition / leaf lists.
  uint32_t err = 0;
  NodeRec* next = a.nodes[parity ^ 1];
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const NodeRec node = a.nodes[parity][i];
    const uint32_t t = node.tree;
    TreeNodeOut* tn = a.tree_nodes + size_t(t) * a.max_tree_nodes;
    const bool acc = a.scratch_flags[i] != 0;
    if (acc) {
      const SplitRec b = a.partial[size_t(i) * a.n_fchunks];
      const uint32_t k = a.scratch_prefix[i];
      const uint32_t kt = k - tree_acc_base[t];
      atomicAdd(&tree_acc[t], 1u);
      const uint32_t li = a.trees[t].n_tree_nodes + 2 * kt, ri = li + 1;
      if (ri >= a.max_tree_nodes) {
        err |= kErrCapacity;
        continue;
      }
      double lv = 0.0, rv = 0.0;
      if (!bounded_leaf(P, b.lg, b.lh, b.ll, b.lu, &lv)) err |= kErrNonFinite;
      if (!bounded_leaf(P, b.rg, b.rh, b.rl, b.ru, &rv)) err |= kErrNonFinite;
      write_leaf(&tn[li], lv);
      write_leaf(&tn[ri], rv);
      TreeNodeOut& pn = tn[node.node_index];
      pn.feature_index = b.feature;
      pn.threshold_bin = b.threshold;
      pn.left_child = li;
      pn.right_child = ri;
      pn.leaf_value = 0.0;
      pn.gain = b.gain;
      pn.default_left = uint8_t(b.default_left);
      pn.flags = 0;
      if (b.lcount + b.rcount != node.seg_cnt) err |= kErrPartition;
      if (!last) {
        const bool build_left = b.lcount <= b.rcount;
        const uint32_t new_slot = a.free_stack[free_top - 1 - k];
        NodeRec L, R;
        L.seg_off = node.seg_off;
        L.seg_cnt = uint32_t(b.lcount);
        R.seg_off = node.seg_off + uint32_t(b.lcount);
        R.seg_cnt = uint32_t(b.rcount);
        L.node_index = li;
        R.node_index = ri;
        L.slot = build_left ? new_slot : node.slot;
        R.slot = build_left ? node.slot : new_slot;
        L.count = b.lcount;
        R.count = b.rcount;
        L.qg = b.lqg;
        L.qh = b.lqh;
        R.qg = b.rqg;
        R.qh = b.rqh;
        L.g = b.lg;
        L.h = b.lh;
        R.g = b.rg;
        R.h = b.rh;
        L.lo = b.ll;
        L.hi = b.lu;
        R.lo = b.rl;
        R.hi = b.ru;
        L.tree = R.tree = t;
        L.depth = R.depth = node.depth + 1;
        // The sibling of the built child keeps the parent's slot; u8 datasets subtract in
        // the next level's split scan (fused_sub), wide ones with subtract_kernel.
        L.sub_from = (a.fused_sub && !build_left) ? new_slot + 1 : 0;
        R.sub_from = (a.fused_sub && build_left) ? new_slot + 1 : 0;
        next[2 * k] = L;
        next[2 * k + 1] = R;
        for (uint32_t w = 0; w < W; ++w) {
          uint32_t path = a.node_path[parity][i * W + w];
          if ((b.feature >> 5) == w) path |= 1u << (b.feature & 31);
          a.node_path[parity ^ 1][(2 * k) * W + w] = path;
          a.node_path[parity ^ 1][(2 * k + 1) * W + w] = path;
        }
        for (uint32_t w = 0; w < W; ++w) {
          uint32_t allowed = 0xffffffffu;
          if (P.n_groups > 0) {  // InteractionAllowsFeature (tree_interactions.cpp:32-45)
            allowed = 0;
            for (uint32_t g = 0; g < P.n_groups; ++g) {
              bool subset = true;
              for (uint32_t u = 0; u < W && subset; ++u) {
                const uint32_t gm = a.group_masks[g * W + u];
                subset = (a.node_path[parity ^ 1][(2 * k) * W + u] & ~gm) == 0;
              }
              if (subset) allowed |= a.group_masks[g * W + w];
            }
          }
          if (a.tree_feature_masks != nullptr) allowed &= a.tree_feature_masks[t * W + w];
          a.node_allowed[parity ^ 1][(2 * k) * W + w] = allowed;
          a.node_allowed[parity ^ 1][(2 * k + 1) * W + w] = allowed;
        }
        BuildEntry be;
        be.tree = t;
        be.parity = uint32_t(parity ^ 1);
        be.seg_off = build_left ? L.seg_off : R.seg_off;
        be.seg_cnt = build_left ? L.seg_cnt : R.seg_cnt;
        be.slot = new_slot;
        be.pad = 0;
        a.build[k] = be;
        SubEntry se;
        se.parent_slot = node.slot;
        se.built_slot = new_slot;
        a.sub[k] = se;
        PartEntry pe;
        pe.tree = t;
        pe.parity = uint32_t(parity);
        pe.seg_off = node.seg_off;
        pe.seg_cnt = node.seg_cnt;
        pe.feature = b.feature;
        pe.threshold = b.threshold;
        pe.default_left = b.default_left;
        pe.lcount = uint32_t(b.lcount);
        a.part[k] = pe;
      }
      if (last) {
        // leaf segment index: number of leaf segments before node i in this level
        // equals i (every node of the last level produces one).
        LeafSeg ls;
        ls.tree = t;
        ls.parity = uint32_t(parity);
        ls.seg_off = node.seg_off;
        ls.seg_cnt = node.seg_cnt;
        ls.split = 1;
        ls.feature = b.feature;
        ls.threshold = b.threshold;
        ls.default_left = b.default_left;
        ls.value = 0.0;
        ls.left_value = lv;
        ls.right_value = rv;
        if (leafseg_base + i < a.max_leafsegs) a.leafseg[leafseg_base + i] = ls;
        else err |= kErrCapacity;
      }
    } else {
      // Node stays a leaf: its rows keep the current leaf value.
      const uint32_t before_acc = a.scratch_prefix[i];
      const uint32_t idx = last ? i : (i - before_acc);  // leaf segments before i
      LeafSeg ls;
      ls.tree = t;
      ls.parity = uint32_t(parity);
      ls.seg_off = node.seg_off;
      ls.seg_cnt = node.seg_cnt;
      ls.split = 0;
      ls.feature = ls.threshold = ls.default_left = 0;
      ls.value = tn[node.node_index].leaf_value;
      ls.left_value = ls.right_value = 0.0;
      if (leafseg_base + idx < a.max_leafsegs) a.leafseg[leafseg_base + idx] = ls;
      else err |= kErrCapacity;
    }
  }
  __syncthreads();
  // Phase C: free slots of nodes that stopped (non-last levels), counters.
  if (!last) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      if (!a.scratch_flags[i]) {
        const uint32_t j = a.scratch_aux[i];
        a.free_stack[free_top - n_acc + j] = a.nodes[parity][i].slot;
      }
    }
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < a.n_trees; t += blockDim.x) {
    a.trees[t].n_tree_nodes += 2 * tree_acc[t];
    a.trees[t].leaf_count += tree_acc[t];
  }
  if (err) raise(ctl, err);
  if (threadIdx.x == 0) {
    const uint32_t n_leafseg_level = carry6[3];
    ctl->n_leafseg = leafseg_base + n_leafseg_level;
    ctl->leaf_chunks = leafchunk_base + carry6[4];
    if (leafseg_base + n_leafseg_level <= a.max_leafsegs)
      a.leaf_prefix[leafseg_base + n_leafseg_level] = leafchunk_base + carry6[4];
    if (last) {
      ctl->n_nodes = 0;
      ctl->n_build = 0;
      ctl->n_sub = 0;
      ctl->n_part = 0;
      ctl->hist_items = 0;
      ctl->part_chunks = 0;
      ctl->split_items = 0;
    } else {
      ctl->free_top = free_top - n_acc + (n - n_acc);
      ctl->n_nodes = 2 * n_acc;
      ctl->n_build = n_acc;
      ctl->n_sub = n_acc;
      ctl->n_part = n_acc;
      a.build_prefix[n_acc] = carry6[1];
      a.part_prefix[n_acc] = carry6[2];
      ctl->hist_items = carry6[1] * a.nfb;
      ctl->part_chunks = carry6[2];
      ctl->split_items = 2 * n_acc * a.n_fchunks;
      ctl->item_rows = item_rows;
    }
    ctl->hist_counter = 0;
  }
}

// ------------------------------------------------------------------------------------
// Partition
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t find_entry(const uint32_t* prefix, uint32_t n, uint32_t c) {
  uint32_t lo = 0, hi = n;  // last entry with prefix <= c
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (prefix[mid] <= c) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ bool row_goes_left(const TrainerDev& a, uint32_t row, uint32_t f,
                                              uint32_t thr, uint32_t dl) {
  // Feature-major copy: a node's rows are sorted, so neighbouring rows share sectors.
  uint32_t b, missing_slot;
  if (a.bins16_fm) {  // wide dataset (launch-uniform)
    b = a.bins16_fm[size_t(f) * a.n_rows + row];
    missing_slot = a.slots - 1;
  } else {
    b = a.bins_fm[size_t(f) * a.n_rows + row];
    missing_slot = kMissingSlot;
  }
  if (a.has_missing[f] && b == missing_slot) return dl != 0;
  return b <= thr;
}

constexpr int kPartThreads = 512;
constexpr int kPartPerThread = kPartChunk / kPartThreads;  // 8

__global__ void __launch_bounds__(kPartThreads) partition_count_kernel(TrainerDev a) {
  __shared__ uint32_t warp_counts[kPartThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t c = blockIdx.x; c < a.ctl->part_chunks; c += gridDim.x) {
    const uint32_t e = find_entry(a.part_prefix, a.ctl->n_part, c);
    const PartEntry pe = a.part[e];
    const uint32_t lc = c - a.part_prefix[e];
    const uint32_t start = lc * kPartChunk;
    const uint32_t count = min(kPartChunk, pe.seg_cnt - start);
    const uint32_t* rows = a.rows + (size_t(pe.tree) * 2 + pe.parity) * a.seg_stride + pe.seg_off + start;
    uint32_t mine = 0;
    // All row ids, then all bin gathers, then the stores: nothing in flight waits on a
    // store that might alias it.
    uint32_t r[kPartPerThread];
#pragma unroll
    for (int k = 0; k < kPartPerThread; ++k) {
      const uint32_t p = uint32_t(k * kPartThreads) + threadIdx.x;
      r[k] = p < count ? __ldg(rows + p) : 0xffffffffu;
    }
    bool left[kPartPerThread];
#pragma unroll
    for (int k = 0; k < kPartPerThread; ++k)
      left[k] = r[k] < a.n_rows && row_goes_left(a, r[k], pe.feature, pe.threshold, pe.default_left);
#pragma unroll
    for (int k = 0; k < kPartPerThread; ++k) {
      const uint32_t word = __ballot_sync(0xffffffffu, left[k]);
      if (lane == 0) a.part_flags[size_t(c) * (kPartChunk / 32) + k * (kPartThreads / 32) + warp] = word;
      mine += left[k];
    }
    for (int off = 16; off > 0; off >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, off);
    if (lane == 0) warp_counts[warp] = mine;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t s = 0;
      for (int w = 0; w < kPartThreads / 32; ++w) s += warp_counts[w];
      a.part_counts[c] = s;
    }
    __syncthreads();
  }
}

// Exclusive prefix of the chunk counts of each partitioned node.
__global__ void __launch_bounds__(1024) partition_scan_kernel(TrainerDev a) {
  __shared__ uint32_t sh[33];
  uint32_t err = 0;
  for (uint32_t e = blockIdx.x; e < a.ctl->n_part; e += gridDim.x) {
    const uint32_t c0 = a.part_prefix[e], c1 = a.part_prefix[e + 1];
    uint32_t carry = 0;
    for (uint32_t base = c0; base < c1; base += blockDim.x) {
      const uint32_t c = base + threadIdx.x;
      uint32_t v[1] = {c < c1 ? a.part_counts[c] : 0u};
      uint32_t tot[1];
      block_scan<1>(v, tot, sh);
      if (c < c1) a.part_offsets[c] = carry + v[0];
      carry += tot[0];
    }
    if (carry != a.part[e].lcount) err |= kErrPartition;
    if (threadIdx.x == 0) atomicAdd(&a.ctl->rows_partitioned, (unsigned long long)a.part[e].seg_cnt);
    __syncthreads();
  }
  if (err && threadIdx.x == 0) raise(a.ctl, err);
}

__global__ void __launch_bounds__(kPartThreads) partition_scatter_kernel(TrainerDev a) {
  constexpr int kWords = kPartChunk / 32;  // 128
  __shared__ uint32_t word_prefix[kWords];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t err = 0;
  for (uint32_t c = blockIdx.x; c < a.ctl->part_chunks; c += gridDim.x) {
    const uint32_t e = find_entry(a.part_prefix, a.ctl->n_part, c);
    const PartEntry pe = a.part[e];
    const uint32_t lc = c - a.part_prefix[e];
    const uint32_t start = lc * kPartChunk;
    const uint32_t count = min(kPartChunk, pe.seg_cnt - start);
    const uint32_t* flags = a.part_flags + size_t(c) * kWords;
    // Exclusive prefix of the word popcounts, in position order.
    if (warp == 0) {
      uint32_t cnt[4], s = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        cnt[q] = __popc(flags[lane * 4 + q]);
        s += cnt[q];
      }
      uint32_t x = s;
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
      }
      uint32_t run = x - s;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        word_prefix[lane * 4 + q] = run;
        run += cnt[q];
      }
    }
    __syncthreads();
    const size_t src_off = (size_t(pe.tree) * 2 + pe.parity) * a.seg_stride + pe.seg_off + start;
    const size_t dst_off = (size_t(pe.tree) * 2 + (pe.parity ^ 1)) * a.seg_stride + pe.seg_off;
    const uint32_t* src = a.rows + src_off;
    uint32_t* dst = a.rows + dst_off;
    const float2* gh_src = a.gh_ordered ? a.gh + src_off : nullptr;
    float2* gh_dst = a.gh_ordered ? a.gh + dst_off : nullptr;
    const uint32_t left_before_chunk = a.part_offsets[c];
    const uint32_t right_before_chunk = start - left_before_chunk;
    // Loads first (flag words, row ids, g/h), then the stores.
    uint32_t word[kPartPerThread], r[kPartPerThread];
    float2 g[kPartPerThread];
#pragma unroll
    for (int k = 0; k < kPartPerThread; ++k) {
      const uint32_t p = uint32_t(k * kPartThreads) + threadIdx.x;
      word[k] = __ldg(flags + k * (kPartThreads / 32) + warp);
      r[k] = p < count ? __ldg(src + p) : 0u;
      g[k] = (p < count && a.gh_ordered) ? __ldg(gh_src + p) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < kPartPerThread; ++k) {
      const uint32_t p = uint32_t(k * kPartThreads) + threadIdx.x;
      const int wi = k * (kPartThreads / 32) + warp;
      if (p < count) {
        const uint32_t below = __popc(word[k] & ((1u << lane) - 1u));
        const uint32_t lpos = word_prefix[wi] + below;  // left rows before p in the chunk
        const bool left = (word[k] >> lane) & 1u;
        const uint32_t rel = left ? left_before_chunk + lpos : pe.lcount + right_before_chunk + (p - lpos);
        if (rel < pe.seg_cnt) {  // always true when the counts agree
          dst[rel] = r[k];
          if (a.gh_ordered) gh_dst[rel] = g[k];
        } else {
          err = kErrPartition;
        }
      }
    }
    __syncthreads();
  }
  if (err) raise(a.ctl, err);
}

// ------------------------------------------------------------------------------------
// Leaf-wise growth (TrainLeafWiseRegressionTree, tree_leafwise.cpp:56-142)
//
// Each step splits, in every tree, the active leaf with the largest gain (the smaller
// node index on equal gains); leaves at max_depth stay active but never split. A leaf's
// best split depends only on its rows, so it is scanned once, when the leaf is created
// (in fixed point the reference's re-evaluation reproduces the same split exactly). A
// step is: select (this kernel: choose, ApplySplit, children, work lists), partition of
// the chosen leaves, histogram of each smaller child, subtraction for its sibling, split
// scan of the children, merge (the children's best splits into the active lists).
// ------------------------------------------------------------------------------------
__device__ SplitRec merged_split(const TrainerDev& a, uint32_t i) {
  SplitRec b = a.partial[size_t(i) * a.n_fchunks];
  for (uint32_t c = 1; c < a.n_fchunks; ++c) {
    const SplitRec x = a.partial[size_t(i) * a.n_fchunks + c];
    if (better_split(x, b)) b = x;
  }
  return b;
}

__device__ __forceinline__ SplitRec no_split() {
  SplitRec b;
  b.gain = 0.0;
  b.valid = 0;
  b.feature = b.threshold = 0;
  b.default_left = 1;
  return b;
}

// Root of every tree becomes its first active leaf (after the level-0 split scan).
__global__ void leafwise_init_kernel(TrainerDev a) {
  const TreeParams& P = a.params;
  const uint32_t W = P.path_words, T = a.n_trees, S = a.lw_slot_cap;
  for (uint32_t t = threadIdx.x; t < T; t += blockDim.x) {
    // Slot t holds the root (round_setup); the tree's other slots form its stack.
    for (uint32_t j = 0; j < S; ++j) a.lw_slots[size_t(t) * S + j] = T + t * S + j;
    a.lw_slot_top[t] = S;
    LeafActive r;
    r.node = a.nodes[0][t];
    r.best = P.max_depth > 0 ? merged_split(a, t) : no_split();
    r.parity = 0;
    r.scanned = 1;
    a.lw_active[size_t(t) * a.lw_cap] = r;
    for (uint32_t w = 0; w < W; ++w) {
      a.lw_path[size_t(t) * a.lw_cap * W + w] = 0;
      a.lw_allowed[size_t(t) * a.lw_cap * W + w] = a.node_allowed[0][t * W + w];
    }
    a.lw_count[t] = 1;
    a.lw_done[t] = 0;
  }
}

__global__ void __launch_bounds__(1024) leafwise_select_kernel(TrainerDev a) {
  __shared__ uint32_t sh[33 * 3];
  __shared__ unsigned long long built_rows;
  const TreeParams& P = a.params;
  const uint32_t W = P.path_words, cap = a.lw_cap, S = a.lw_slot_cap;
  const uint32_t t = threadIdx.x;
  if (t == 0) built_rows = 0;
  __syncthreads();
  uint32_t err = 0;
  bool split = false, build = false;
  uint32_t n_scan = 0, kid_at[2] = {0, 0};
  PartEntry pe{};
  BuildEntry be{};
  SubEntry se{};
  if (t < a.n_trees && !a.lw_done[t]) {
    LeafActive* act = a.lw_active + size_t(t) * cap;
    uint32_t* path = a.lw_path + size_t(t) * cap * W;
    uint32_t* allowed = a.lw_allowed + size_t(t) * cap * W;
    TreeState& ts = a.trees[t];
    const uint32_t cnt = a.lw_count[t];
    int best = -1;
    if (cnt > a.lw_max_active) {
      err |= kErrLeafQueue;
    } else if (ts.leaf_count < a.lw_max_leaves) {
      for (uint32_t j = 0; j < cnt; ++j) {  // IsBetterLeafWiseCandidate (tree_leafwise.cpp:16-27)
        const LeafActive& l = act[j];
        if (l.node.depth >= P.max_depth || !l.scanned || !l.best.valid) continue;
        if (best < 0 || l.best.gain > act[best].best.gain ||
            (l.best.gain == act[best].best.gain && l.node.node_index < act[best].node.node_index))
          best = int(j);
      }
    }
    if (best < 0) {
      a.lw_done[t] = 1;
    } else {
      const LeafActive c = act[best];
      const SplitRec& b = c.best;
      TreeNodeOut* tn = a.tree_nodes + size_t(t) * a.max_tree_nodes;
      const uint32_t li = ts.n_tree_nodes, ri = li + 1;
      const uint32_t depth = c.node.depth + 1;
      const bool grow = depth < P.max_depth;
      if (ri >= a.max_tree_nodes || cnt + 2 > cap || (grow && a.lw_slot_top[t] == 0)) {
        err |= kErrCapacity;
        a.lw_done[t] = 1;
      } else {
        // ApplySplit (tree_structure.cpp:118-148).
        double lv = 0.0, rv = 0.0;
        if (!bounded_leaf(P, b.lg, b.lh, b.ll, b.lu, &lv)) err |= kErrNonFinite;
        if (!bounded_leaf(P, b.rg, b.rh, b.rl, b.ru, &rv)) err |= kErrNonFinite;
        write_leaf(&tn[li], lv);
        write_leaf(&tn[ri], rv);
        TreeNodeOut& pn = tn[c.node.node_index];
        pn.feature_index = b.feature;
        pn.threshold_bin = b.threshold;
        pn.left_child = li;
        pn.right_child = ri;
        pn.leaf_value = 0.0;
        pn.gain = b.gain;
        pn.default_left = uint8_t(b.default_left);
        pn.flags = 0;
        ts.n_tree_nodes += 2;
        ts.leaf_count += 1;
        if (b.lcount + b.rcount != c.node.seg_cnt) err |= kErrPartition;
        // Children in the other row buffer: left rows, then right rows (the partition).
        const uint32_t np = c.parity ^ 1u;
        const bool build_left = b.lcount <= b.rcount;
        uint32_t new_slot = 0xffffffffu;
        if (grow) new_slot = a.lw_slots[size_t(t) * S + --a.lw_slot_top[t]];
        else a.lw_slots[size_t(t) * S + a.lw_slot_top[t]++] = c.node.slot;  // no child histograms
        LeafActive kid[2];
        for (int k = 0; k < 2; ++k) {
          NodeRec& n = kid[k].node;
          const bool left = k == 0;
          n.seg_off = left ? c.node.seg_off : c.node.seg_off + uint32_t(b.lcount);
          n.seg_cnt = uint32_t(left ? b.lcount : b.rcount);
          n.node_index = left ? li : ri;
          n.slot = !grow ? 0xffffffffu : ((left == build_left) ? new_slot : c.node.slot);
          n.count = left ? b.lcount : b.rcount;
          n.qg = left ? b.lqg : b.rqg;
          n.qh = left ? b.lqh : b.rqh;
          n.g = left ? b.lg : b.rg;
          n.h = left ? b.lh : b.rh;
          n.lo = left ? b.ll : b.rl;
          n.hi = left ? b.lu : b.ru;
          n.tree = t;
          n.depth = depth;
          n.sub_from = 0;  // leaf-wise steps subtract with subtract_kernel
          kid[k].best = no_split();
          kid[k].parity = np;
          kid[k].scanned = grow ? 0u : 1u;
        }
        // Children's path and allowed words go to positions cnt, cnt + 1 (free), the
        // chosen leaf's place takes the last leaf, then the children move down by one.
        for (int k = 0; k < 2; ++k)
          for (uint32_t w = 0; w < W; ++w) {
            uint32_t pw = path[size_t(best) * W + w];
            if ((b.feature >> 5) == w) pw |= 1u << (b.feature & 31);
            path[size_t(cnt + k) * W + w] = pw;
          }
        for (uint32_t w = 0; w < W; ++w) {
          uint32_t al = 0xffffffffu;
          if (P.n_groups > 0) {  // InteractionAllowsFeature (tree_interactions.cpp:32-45)
            al = 0;
            for (uint32_t g = 0; g < P.n_groups; ++g) {
              bool subset = true;
              for (uint32_t u = 0; u < W && subset; ++u)
                subset = (path[size_t(cnt) * W + u] & ~a.group_masks[g * W + u]) == 0;
              if (subset) al |= a.group_masks[g * W + w];
            }
          }
          if (a.tree_feature_masks != nullptr) al &= a.tree_feature_masks[t * W + w];
          allowed[size_t(cnt) * W + w] = al;
          allowed[size_t(cnt + 1) * W + w] = al;
        }
        const uint32_t last = cnt - 1;
        if (uint32_t(best) != last) {
          act[best] = act[last];
          for (uint32_t w = 0; w < W; ++w) {
            path[size_t(best) * W + w] = path[size_t(last) * W + w];
            allowed[size_t(best) * W + w] = allowed[size_t(last) * W + w];
          }
        }
        for (int k = 0; k < 2; ++k) {
          act[last + k] = kid[k];
          for (uint32_t w = 0; w < W; ++w) {
            path[size_t(last + k) * W + w] = path[size_t(cnt + k) * W + w];
            allowed[size_t(last + k) * W + w] = allowed[size_t(cnt + k) * W + w];
          }
        }
        a.lw_count[t] = cnt + 1;
        // Room for both children (tree_leafwise.cpp:130-134).
        if (!(cnt - 1 + 2 <= a.lw_max_active || ts.leaf_count >= a.lw_max_leaves)) {
          err |= kErrLeafQueue;
          a.lw_done[t] = 1;
        }
        split = true;
        pe.tree = t;
        pe.parity = c.parity;
        pe.seg_off = c.node.seg_off;
        pe.seg_cnt = c.node.seg_cnt;
        pe.feature = b.feature;
        pe.threshold = b.threshold;
        pe.default_left = b.default_left;
        pe.lcount = uint32_t(b.lcount);
        if (grow) {
          build = true;
          be.tree = t;
          be.parity = np;
          be.seg_off = build_left ? kid[0].node.seg_off : kid[1].node.seg_off;
          be.seg_cnt = build_left ? kid[0].node.seg_cnt : kid[1].node.seg_cnt;
          be.slot = new_slot;
          be.pad = 0;
          se.parent_slot = c.node.slot;
          se.built_slot = new_slot;
          atomicAdd(&built_rows, (unsigned long long)be.seg_cnt);
          n_scan = 2;
          kid_at[0] = last;
          kid_at[1] = last + 1;
        }
      }
    }
  }
  if (err) raise(a.ctl, err);
  uint32_t v[3] = {split ? 1u : 0u, build ? 1u : 0u, n_scan};
  uint32_t tot[3];
  block_scan<3>(v, tot, sh);
  if (split) a.part[v[0]] = pe;
  if (build) {
    a.build[v[1]] = be;
    a.sub[v[1]] = se;
  }
  for (uint32_t k = 0; k < n_scan; ++k) {
    const uint32_t s = v[2] + k;
    a.nodes[1][s] = a.lw_active[size_t(t) * cap + kid_at[k]].node;
    for (uint32_t w = 0; w < W; ++w)
      a.node_allowed[1][size_t(s) * W + w] = a.lw_allowed[(size_t(t) * cap + kid_at[k]) * W + w];
    a.lw_scan_map[s] = (t << 16) | kid_at[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // work lists of the step (few entries: one per tree)
    Control* ctl = a.ctl;
    uint32_t acc = 0;
    for (uint32_t e = 0; e < tot[0]; ++e) {
      a.part_prefix[e] = acc;
      acc += ceil_div(a.part[e].seg_cnt, kPartChunk);
    }
    a.part_prefix[tot[0]] = acc;
    ctl->n_part = tot[0];
    ctl->part_chunks = acc;
    const uint32_t item_rows =
        a.item_rows ? a.item_rows : adaptive_item_rows(built_rows, a.nfb, a.sm_count, a.items_per_sm);
    acc = 0;
    for (uint32_t e = 0; e < tot[1]; ++e) {
      a.build_prefix[e] = acc;
      acc += ceil_div(a.build[e].seg_cnt, item_rows);
    }
    a.build_prefix[tot[1]] = acc;
    ctl->n_build = tot[1];
    ctl->n_sub = tot[1];
    ctl->hist_items = acc * a.nfb;
    ctl->hist_counter = 0;
    ctl->item_rows = item_rows;
    ctl->n_nodes = tot[2];
    ctl->split_items = tot[2] * a.n_fchunks;
  }
}

// The children's best splits into their active entries.
__global__ void leafwise_merge_kernel(TrainerDev a) {
  for (uint32_t s = threadIdx.x; s < a.ctl->n_nodes; s += blockDim.x) {
    const uint32_t m = a.lw_scan_map[s];
    LeafActive& l = a.lw_active[size_t(m >> 16) * a.lw_cap + (m & 0xFFFFu)];
    l.best = merged_split(a, s);
    l.scanned = 1;
  }
}

// Every active leaf becomes a leaf segment of the prediction update.
__global__ void leafwise_finish_kernel(TrainerDev a) {
  if (threadIdx.x != 0) return;
  Control* ctl = a.ctl;
  uint32_t n = 0, chunks = 0, err = 0;
  for (uint32_t t = 0; t < a.n_trees; ++t) {
    const LeafActive* act = a.lw_active + size_t(t) * a.lw_cap;
    const TreeNodeOut* tn = a.tree_nodes + size_t(t) * a.max_tree_nodes;
    for (uint32_t j = 0; j < a.lw_count[t]; ++j) {
      if (n >= a.max_leafsegs) {
        err |= kErrCapacity;
        break;
      }
      LeafSeg ls;
      ls.tree = t;
      ls.parity = act[j].parity;
      ls.seg_off = act[j].node.seg_off;
      ls.seg_cnt = act[j].node.seg_cnt;
      ls.split = 0;
      ls.feature = ls.threshold = ls.default_left = 0;
      ls.value = tn[act[j].node.node_index].leaf_value;
      ls.left_value = ls.right_value = 0.0;
      a.leafseg[n] = ls;
      a.leaf_prefix[n] = chunks;
      chunks += ceil_div(ls.seg_cnt, kApplyChunk);
      ++n;
    }
  }
  a.leaf_prefix[n] = chunks;
  ctl->n_leafseg = n;
  ctl->leaf_chunks = chunks;
  ctl->n_nodes = ctl->n_build = ctl->n_sub = ctl->n_part = 0;
  ctl->hist_items = ctl->part_chunks = ctl->split_items = 0;
  if (err) raise(ctl, err);
}

// ------------------------------------------------------------------------------------
// Leaf application and round end
// ------------------------------------------------------------------------------------
// The prediction update runs in two passes. The first walks the leaf segments (a
// segment's rows ascend but are spread over the whole row range), routes the rows of
// last-level splits, and records per row which of its segment's steps applies (a 4-byte
// scattered write into an array that stays in L2); the second walks the rows in order and
// adds that step to the row's prediction, so the FP64 predictions are read and written as
// streams instead of one 32-byte sector each way per row.
constexpr uint32_t kNoLeaf = 0xffffffffu;

__global__ void __launch_bounds__(256, 4) apply_leaves_kernel(TrainerDev a) {
  if (a.skip_apply) return;  // forest trees: no training predictions
  const double lr = a.params.learning_rate;
  uint32_t err = 0;
  const uint32_t n_seg = a.ctl->n_leafseg;
  const uint32_t chunks = a.ctl->leaf_chunks;
  for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
    const uint32_t s = find_entry(a.leaf_prefix, n_seg, c);
    const LeafSeg ls = a.leafseg[s];
    const uint32_t start = (c - a.leaf_prefix[s]) * kApplyChunk;
    const uint32_t count = min(kApplyChunk, ls.seg_cnt - start);
    const uint32_t* rows = a.rows + (size_t(ls.tree) * 2 + ls.parity) * a.seg_stride + ls.seg_off + start;
    uint32_t* leaf_of = a.leaf_of + size_t(ls.tree) * a.n_rows;
    if (start == 0 && threadIdx.x == 0) {
      // lr * leaf is the same product for every row of a leaf.
      const double step = __dmul_rn(lr, ls.value);
      a.leaf_steps[2 * s] = ls.split ? __dmul_rn(lr, ls.left_value) : step;
      a.leaf_steps[2 * s + 1] = ls.split ? __dmul_rn(lr, ls.right_value) : step;
    }
    // Eight rows per thread at a time: row ids, then the routing gathers, then the stores.
    constexpr int B = 8;
    for (uint32_t p0 = 0; p0 < count; p0 += B * blockDim.x) {
      uint32_t r[B];
#pragma unroll
      for (int k = 0; k < B; ++k) {
        const uint32_t p = p0 + k * blockDim.x + threadIdx.x;
        r[k] = p < count ? __ldg(rows + p) : kNoLeaf;
      }
      uint32_t side[B];
#pragma unroll
      for (int k = 0; k < B; ++k)
        side[k] = (ls.split && r[k] < a.n_rows &&
                   !row_goes_left(a, r[k], ls.feature, ls.threshold, ls.default_left)) ? 1u : 0u;
#pragma unroll
      for (int k = 0; k < B; ++k) {
        const uint32_t p = p0 + k * blockDim.x + threadIdx.x;
        if (p >= count) continue;
        if (r[k] >= a.n_rows) {
          err = kErrCapacity;
          continue;
        }
        leaf_of[r[k]] = 2 * s + side[k];
      }
    }
  }
  if (err) raise(a.ctl, err);
}

// Row order: prediction += the step recorded for the row, then the record is cleared, so
// a row that no leaf segment covered in a round is caught in the next.
__global__ void __launch_bounds__(256) apply_steps_kernel(TrainerDev a) {
  if (a.skip_apply) return;
  uint32_t err = 0;
  const uint32_t steps = 2 * a.ctl->n_leafseg;
  // Softmax trees update the margins of the current round's class.
  const uint32_t klass = a.n_classes ? *a.round_counter % a.n_classes : 0u;
  const size_t total = size_t(a.n_trees) * a.n_rows;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const uint32_t t = uint32_t(i / a.n_rows);
    const uint32_t r = uint32_t(i - size_t(t) * a.n_rows);
    const uint32_t idx = a.leaf_of[i];
    if (idx >= steps) {
      err = kErrPartition;
      continue;
    }
    a.leaf_of[i] = kNoLeaf;
    double* pred = a.preds + size_t(a.n_classes ? klass : t) * a.n_rows;
    const double out = __dadd_rn(pred[r], a.leaf_steps[idx]);
    if (!f64_finite(out)) err = kErrNonFinite;
    pred[r] = out;
  }
  if (err) raise(a.ctl, err);
}

__global__ void round_end_kernel(TrainerDev a) {
  const uint32_t round = *a.round_counter;
  if (round >= a.max_rounds) {
    if (threadIdx.x == 0) raise(a.ctl, kErrCapacity);
    return;
  }
  for (uint32_t t = 0; t < a.n_trees; ++t) {
    const uint32_t cnt = a.trees[t].n_tree_nodes;
    const TreeNodeOut* src = a.tree_nodes + size_t(t) * a.max_tree_nodes;
    TreeNodeOut* dst = a.model_nodes + (size_t(round) * a.n_trees + t) * a.max_tree_nodes;
    for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) dst[i] = src[i];
    if (threadIdx.x == 0) a.model_counts[size_t(round) * a.n_trees + t] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) *a.round_counter = round + 1;
}

// ------------------------------------------------------------------------------------
// Standalone entries
// ------------------------------------------------------------------------------------
__global__ void squared_error_kernel(const double* labels, const double* preds, uint64_t n,
                                     double* out, uint32_t* error) {
  uint32_t bad = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
       i += uint64_t(gridDim.x) * blockDim.x) {
    const double y = labels[i], p = preds[i];
    const double g = __dadd_rn(p, -y);
    if (!isfinite(y) || !isfinite(p) || !isfinite(g)) bad = 1;
    out[2 * i] = g;
    out[2 * i + 1] = 1.0;
  }
  if (bad) atomicOr(error, kErrGradient);
}

// RegressionModel::Predict (trainer.cpp:268-282): per row, trees in order,
// result += lr * leaf; traversal of RegressionTree::Predict (tree.cpp:179-214).
// BinT: u8 bins (missing rows at 255) or u16 bins of a wide dataset (at missing_slot).
template <typename BinT>
__global__ void predict_kernel(const BinT* bins_fm, uint32_t missing_slot, uint32_t n_rows,
                               const uint8_t* has_missing, const TreeNodeOut* nodes,
                               const uint32_t* tree_offsets, uint32_t n_trees, double base,
                               double lr, double* out, uint32_t* error) {
  uint32_t bad = 0;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) {
    double acc = base;
    for (uint32_t t = 0; t < n_trees; ++t) {
      const TreeNodeOut* tn = nodes + tree_offsets[t];
      const uint32_t size = tree_offsets[t + 1] - tree_offsets[t];
      uint32_t node = 0, visited = 0;
      for (;;) {
        if (node >= size || ++visited > size) {
          bad = 1;
          break;
        }
        const TreeNodeOut nd = tn[node];
        if (nd.flags & 1u) {
          acc = __dadd_rn(acc, __dmul_rn(lr, nd.leaf_value));
          break;
        }
        const uint32_t f = nd.feature_index;
        const uint32_t b = bins_fm[size_t(f) * n_rows + r];
        const bool left = (has_missing[f] && b == missing_slot) ? nd.default_left != 0
                                                                : b <= nd.threshold_bin;
        node = left ? nd.left_child : nd.right_child;
      }
    }
    out[r] = acc;
  }
  if (bad) atomicOr(error, kErrCapacity);
}

// Feature-major [features][rows] bins (u8 or u16) + optional missing mask -> three u8
// layouts with missing rows at 255: rows padded to nfb * 32 bytes and column blocks
// [nfb][rows][32] (histograms of sparse and dense levels), and a feature-major copy (row
// routing). Out-of-range bins set bit 0 of `error`.
// Feature block fb0 + blockIdx.y of the dataset. `src` and `missing` hold the features from
// src_f0 on (the whole matrix: src_f0 = 0; one staged feature block: src_f0 = 32 * fb0).
__global__ void pack_bins_kernel(const void* src, uint32_t width, const uint8_t* missing,
                                 const uint32_t* bin_count, uint32_t n_rows, uint32_t features,
                                 uint32_t nfb, uint8_t* out, uint8_t* out_blocked,
                                 uint8_t* out_fm, uint32_t* error, uint32_t fb0, uint32_t src_f0) {
  __shared__ uint8_t tile[32][129];
  const uint32_t fb = fb0 + blockIdx.y;
  uint32_t bad = 0;
  for (uint32_t r0 = blockIdx.x * 128; r0 < n_rows; r0 += gridDim.x * 128) {
    // load 32 features x 128 rows (coalesced along rows)
    if (width == 1 && n_rows % 16 == 0 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0 &&
        (reinterpret_cast<uintptr_t>(missing) & 15u) == 0) {
      // Sixteen rows per thread: 8 threads read one feature's 128 rows, a warp four
      // features (four 128-byte requests per instruction).
      for (uint32_t k = threadIdx.x; k < 32 * 8; k += blockDim.x) {
        const uint32_t c = k / 8, r = (k % 8) * 16;
        const uint32_t f = fb * 32 + c, row = r0 + r;
        uint4 out4 = make_uint4(0, 0, 0, 0);
        if (f < features && row < n_rows) {  // n_rows % 16 == 0: all sixteen rows exist
          const size_t idx = size_t(f) * n_rows + row, sidx = size_t(f - src_f0) * n_rows + row;
          const uint4 b16 = *reinterpret_cast<const uint4*>(static_cast<const uint8_t*>(src) + sidx);
          const uint4 m16 = missing ? *reinterpret_cast<const uint4*>(missing + sidx) : make_uint4(0, 0, 0, 0);
          const uint32_t nb = bin_count[f];
          const uint32_t bw[4] = {b16.x, b16.y, b16.z, b16.w}, mw[4] = {m16.x, m16.y, m16.z, m16.w};
          uint32_t ow[4];
#pragma unroll
          for (uint32_t j = 0; j < 4; ++j) {
            uint32_t word = 0;
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
              const uint32_t b = (bw[j] >> (8 * q)) & 0xFFu;
              uint32_t v;
              if ((mw[j] >> (8 * q)) & 0xFFu) {
                if (nb > 255) bad = 1;
                v = kMissingSlot;
              } else {
                if (b >= nb) bad = 1;
                v = b;
              }
              tile[c][r + 4 * j + q] = uint8_t(v);
              word |= v << (8 * q);
            }
            ow[j] = word;
          }
          out4 = make_uint4(ow[0], ow[1], ow[2], ow[3]);
          *reinterpret_cast<uint4*>(out_fm + idx) = out4;
        } else {
#pragma unroll
          for (uint32_t q = 0; q < 16; ++q) tile[c][r + q] = 0;
        }
      }
    } else if (width == 1 && n_rows % 4 == 0 && (reinterpret_cast<uintptr_t>(src) & 3u) == 0 &&
               (reinterpret_cast<uintptr_t>(missing) & 3u) == 0) {
      // Four rows per thread: a warp reads one feature's 128 rows as one 128-byte request
      // (the source may be page-locked host memory read over the host link).
      for (uint32_t k = threadIdx.x; k < 32 * 32; k += blockDim.x) {
        const uint32_t c = k / 32, r = (k % 32) * 4;
        const uint32_t f = fb * 32 + c, row = r0 + r;
        uint32_t word = 0;
        if (f < features && row < n_rows) {  // n_rows % 4 == 0: all four rows exist
          const size_t idx = size_t(f) * n_rows + row, sidx = size_t(f - src_f0) * n_rows + row;
          const uint32_t b4 = *reinterpret_cast<const uint32_t*>(static_cast<const uint8_t*>(src) + sidx);
          const uint32_t m4 = missing ? *reinterpret_cast<const uint32_t*>(missing + sidx) : 0u;
          const uint32_t nb = bin_count[f];
#pragma unroll
          for (uint32_t q = 0; q < 4; ++q) {
            const uint32_t b = (b4 >> (8 * q)) & 0xFFu;
            uint32_t v;
            if ((m4 >> (8 * q)) & 0xFFu) {
              if (nb > 255) bad = 1;
              v = kMissingSlot;
            } else {
              if (b >= nb) bad = 1;
              v = b;
            }
            tile[c][r + q] = uint8_t(v);
            word |= v << (8 * q);
          }
          *reinterpret_cast<uint32_t*>(out_fm + idx) = word;
        } else {
#pragma unroll
          for (uint32_t q = 0; q < 4; ++q) tile[c][r + q] = 0;
        }
      }
    } else {
      for (uint32_t k = threadIdx.x; k < 32 * 128; k += blockDim.x) {
        const uint32_t c = k / 128, r = k % 128;
        const uint32_t f = fb * 32 + c, row = r0 + r;
        uint8_t v = 0;
        if (f < features && row < n_rows) {
          const size_t sidx = size_t(f - src_f0) * n_rows + row;
          const uint32_t b = width == 1 ? static_cast<const uint8_t*>(src)[sidx]
                                        : static_cast<const uint16_t*>(src)[sidx];
          const bool miss = missing != nullptr && missing[sidx] != 0;
          if (miss) {
            if (bin_count[f] > 255) bad = 1;
            v = uint8_t(kMissingSlot);
          } else {
            if (b >= bin_count[f]) bad = 1;
            v = uint8_t(b);
          }
        }
        tile[c][r] = v;
        if (f < features && row < n_rows) out_fm[size_t(f) * n_rows + row] = v;
      }
    }
    __syncthreads();
    // store 128 rows x 32 bytes: row-major rows padded to nfb * 32 bytes
    for (uint32_t k = threadIdx.x; k < 32 * 128; k += blockDim.x) {
      const uint32_t r = k / 32, c = k % 32;
      const uint32_t row = r0 + r;
      if (row < n_rows) {
        out[size_t(row) * nfb * kBlockFeatures + fb * kBlockFeatures + c] = tile[c][r];
        out_blocked[(size_t(fb) * n_rows + row) * kBlockFeatures + c] = tile[c][r];
      }
    }
    __syncthreads();
  }
  if (bad) atomicOr(error, 1u);
}

// Wide datasets: one feature block fb (features 32 fb .. 32 fb + 31, staged from src, u8 or
// u16, with the optional missing mask) -> the u16 column blocks [nfb][n_rows][32] (histogram
// gathers: a row's block is 64 contiguous bytes) and the feature-major u16 copy (row
// routing), missing rows at slots - 1. Out-of-range bins set bit 0 of `error`.
__global__ void pack_bins16_kernel(const void* src, uint32_t width, const uint8_t* missing,
                                   const uint32_t* bin_count, uint32_t n_rows, uint32_t features,
                                   uint32_t fb, uint32_t slots, uint16_t* out_blocked,
                                   uint16_t* out_fm, uint32_t* error) {
  __shared__ uint16_t tile[32][130];
  uint32_t bad = 0;
  for (uint32_t r0 = blockIdx.x * 128; r0 < n_rows; r0 += gridDim.x * 128) {
    // 32 features x 128 rows, read along rows.
    for (uint32_t k = threadIdx.x; k < 32 * 128; k += blockDim.x) {
      const uint32_t c = k / 128, r = k % 128;
      const uint32_t f = fb * 32 + c, row = r0 + r;
      uint32_t v = 0;
      if (f < features && row < n_rows) {
        const size_t sidx = size_t(c) * n_rows + row;
        const uint32_t b = width == 1 ? static_cast<const uint8_t*>(src)[sidx]
                                      : static_cast<const uint16_t*>(src)[sidx];
        if (missing != nullptr && missing[sidx] != 0) {
          if (bin_count[f] > slots - 1) bad = 1;
          v = slots - 1;
        } else {
          if (b >= bin_count[f]) bad = 1;
          v = b;
        }
        out_fm[size_t(f) * n_rows + row] = uint16_t(v);
      }
      tile[c][r] = uint16_t(v);
    }
    __syncthreads();
    // 128 rows x 32 features: a warp writes one row's 64-byte block.
    for (uint32_t k = threadIdx.x; k < 32 * 128; k += blockDim.x) {
      const uint32_t r = k / 32, c = k % 32;
      const uint32_t row = r0 + r;
      if (row < n_rows) out_blocked[(size_t(fb) * n_rows + row) * 32 + c] = tile[c][r];
    }
    __syncthreads();
  }
  if (bad) atomicOr(error, 1u);
}

}  // namespace

cudaError_t launch_round_begin(const TrainerDev& a, cudaStream_t s) {
  round_begin_kernel<<<1, 1024, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_gradients(const TrainerDev& a, int grid, cudaStream_t s) {
  if (a.objective == 0 && !a.n_classes)  // twice the CTAs: twice as many fit on an SM
    gradients_kernel<true><<<dim3(2 * grid, a.n_trees), 256, 0, s>>>(a);
  else
    gradients_kernel<false><<<dim3(grid, a.n_trees), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_round_setup(const TrainerDev& a, cudaStream_t s) {
  round_setup_kernel<<<1, 1024, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_zero_build_slots(const TrainerDev& a, int grid, cudaStream_t s) {
  zero_build_slots_kernel<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_root_stats(const TrainerDev& a, cudaStream_t s) {
  root_stats_kernel<<<1, 1024, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_root_cache(const TrainerDev& a, int save, int grid, cudaStream_t s) {
  root_cache_kernel<<<grid, 256, 0, s>>>(a, save);
  return cudaGetLastError();
}
cudaError_t launch_subtract(const TrainerDev& a, int grid, cudaStream_t s) {
  subtract_kernel<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}
template <bool FIXED, bool SCREEN, bool WIDE>
cudaError_t launch_scan_shape(const TrainerDev& a, int parity, int grid, int threads, cudaStream_t s) {
  const size_t smem = scan_smem_per_warp<FIXED, SCREEN>() * size_t(threads / 32);
  static std::atomic<unsigned long long> configured{0};  // one bit per device
  const cudaError_t err = opt_in_dynamic_smem(configured, split_scan_kernel<FIXED, SCREEN, WIDE>,
                                              scan_smem_per_warp<FIXED, SCREEN>() * (kScanThreadsMax / 32));
  if (err != cudaSuccess) return err;
  split_scan_kernel<FIXED, SCREEN, WIDE><<<grid, threads, smem, s>>>(a, parity);
  return cudaGetLastError();
}
template <bool FIXED, bool SCREEN>
cudaError_t launch_scan_variant(const TrainerDev& a, int parity, int grid, int threads, cudaStream_t s) {
  if (a.slots == uint32_t(kSlots)) return launch_scan_shape<FIXED, SCREEN, false>(a, parity, grid, threads, s);
  if (a.slots < uint32_t(kSlots) || a.slots % uint32_t(kSlots)) return cudaErrorInvalidValue;
  return launch_scan_shape<FIXED, SCREEN, true>(a, parity, grid, threads, s);
}

uint32_t split_scan_kernels(const TrainerDev& a) {
  return a.node_screen && a.scan_two_phase ? 2u : 1u;
}

cudaError_t launch_split_scan(const TrainerDev& a, int parity, int grid, cudaStream_t s) {
  const int threads = int(a.scan_threads);
  if (threads < 32 || threads > kScanThreadsMax || threads % 32) return cudaErrorInvalidValue;
  const bool fixed = a.mode == kModeFixed;
  if (split_scan_kernels(a) == 2) {
    // node_screen was cleared by the level's zero_build_slots_kernel.
    cudaError_t err;
    // The screen phase holds about half the registers: twice the CTAs.
    err = fixed ? launch_scan_variant<true, true>(a, parity, 2 * grid, threads, s)
                : launch_scan_variant<false, true>(a, parity, 2 * grid, threads, s);
    if (err != cudaSuccess) return err;
  }
  return fixed ? launch_scan_variant<true, false>(a, parity, grid, threads, s)
               : launch_scan_variant<false, false>(a, parity, grid, threads, s);
}
cudaError_t launch_leafwise_init(const TrainerDev& a, cudaStream_t s) {
  leafwise_init_kernel<<<1, 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_leafwise_select(const TrainerDev& a, cudaStream_t s) {
  leafwise_select_kernel<<<1, 1024, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_leafwise_merge(const TrainerDev& a, cudaStream_t s) {
  leafwise_merge_kernel<<<1, 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_leafwise_finish(const TrainerDev& a, cudaStream_t s) {
  leafwise_finish_kernel<<<1, 32, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_finalize(const TrainerDev& a, int parity, uint32_t depth, cudaStream_t s) {
  finalize_kernel<<<1, 1024, 0, s>>>(a, parity, depth);
  return cudaGetLastError();
}
cudaError_t launch_partition(const TrainerDev& a, int grid, cudaStream_t s) {
  partition_count_kernel<<<grid, kPartThreads, 0, s>>>(a);
  partition_scan_kernel<<<grid, 1024, 0, s>>>(a);
  partition_scatter_kernel<<<grid, kPartThreads, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_partition_count(const TrainerDev& a, int grid, cudaStream_t s) {
  partition_count_kernel<<<grid, kPartThreads, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_partition_finish(const TrainerDev& a, int grid, cudaStream_t s) {
  partition_scan_kernel<<<grid, 1024, 0, s>>>(a);
  partition_scatter_kernel<<<grid, kPartThreads, 0, s>>>(a);
  return cudaGetLastError();
}
__global__ void fill_f64_kernel(double* dst, uint64_t n, double value) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    dst[i] = value;
}
cudaError_t launch_fill_f64(double* dst, uint64_t n, double value, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, 4096);
  fill_f64_kernel<<<unsigned(blocks), 256, 0, s>>>(dst, n, value);
  return cudaGetLastError();
}
cudaError_t launch_apply_leaves(const TrainerDev& a, int grid, cudaStream_t s) {
  apply_leaves_kernel<<<grid, 256, 0, s>>>(a);
  apply_steps_kernel<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_round_end(const TrainerDev& a, cudaStream_t s) {
  round_end_kernel<<<1, 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_squared_error(const double* labels, const double* preds, uint64_t n,
                                 double* out, uint32_t* error, cudaStream_t s) {
  const int grid = int(std::min<uint64_t>((n + 255) / 256, 152ull * 16));
  squared_error_kernel<<<grid > 0 ? grid : 1, 256, 0, s>>>(labels, preds, n, out, error);
  return cudaGetLastError();
}
cudaError_t launch_pack_bins(const void* src, uint32_t width, const uint8_t* missing,
                             const uint32_t* bin_count, uint32_t n_rows, uint32_t features,
                             uint32_t nfb, uint8_t* out_rows, uint8_t* out_blocked,
                             uint8_t* out_fm, uint32_t* error, cudaStream_t s) {
  const uint32_t gx = std::min<uint32_t>((n_rows + 127) / 128, 4096u);
  pack_bins_kernel<<<dim3(gx > 0 ? gx : 1, nfb), 256, 0, s>>>(src, width, missing, bin_count,
                                                              n_rows, features, nfb, out_rows,
                                                              out_blocked, out_fm, error, 0u, 0u);
  return cudaGetLastError();
}
cudaError_t launch_pack_bins_block(const void* src_block, uint32_t width, const uint8_t* missing_block,
                                   const uint32_t* bin_count, uint32_t n_rows, uint32_t features,
                                   uint32_t nfb, uint32_t fb, uint8_t* out_rows, uint8_t* out_blocked,
                                   uint8_t* out_fm, uint32_t* error, cudaStream_t s) {
  const uint32_t gx = std::min<uint32_t>((n_rows + 127) / 128, 4096u);
  pack_bins_kernel<<<dim3(gx > 0 ? gx : 1, 1), 256, 0, s>>>(src_block, width, missing_block, bin_count,
                                                            n_rows, features, nfb, out_rows, out_blocked,
                                                            out_fm, error, fb, fb * kBlockFeatures);
  return cudaGetLastError();
}
cudaError_t launch_pack_bins16_block(const void* src_block, uint32_t width,
                                     const uint8_t* missing_block, const uint32_t* bin_count,
                                     uint32_t n_rows, uint32_t features, uint32_t fb,
                                     uint32_t slots, uint16_t* out_blocked, uint16_t* out_fm,
                                     uint32_t* error, cudaStream_t s) {
  if (slots < 2 || slots > 65536) return cudaErrorInvalidValue;
  const uint32_t gx = std::min<uint32_t>((n_rows + 127) / 128, 4096u);
  pack_bins16_kernel<<<gx > 0 ? gx : 1, 256, 0, s>>>(src_block, width, missing_block, bin_count, n_rows,
                                                     features, fb, slots, out_blocked, out_fm, error);
  return cudaGetLastError();
}
cudaError_t launch_predict(const uint8_t* bins_fm, const uint16_t* bins16_fm, uint32_t slots,
                           uint32_t n_rows, uint32_t nfb, const uint8_t* has_missing,
                           const TreeNodeOut* nodes, const uint32_t* tree_offsets,
                           uint32_t n_trees, double base, double lr, double* out,
                           uint32_t* error, cudaStream_t s) {
  (void)nfb;
  const int grid = int(std::min<uint64_t>((n_rows + 255) / 256, 152ull * 16));
  if (bins16_fm) {
    if (slots < 2 || slots > 65536) return cudaErrorInvalidValue;
    predict_kernel<uint16_t><<<grid > 0 ? grid : 1, 256, 0, s>>>(
        bins16_fm, slots - 1, n_rows, has_missing, nodes, tree_offsets, n_trees, base, lr, out, error);
  } else {
    predict_kernel<uint8_t><<<grid > 0 ? grid : 1, 256, 0, s>>>(
        bins_fm, uint32_t(kMissingSlot), n_rows, has_missing, nodes, tree_offsets, n_trees, base,
        lr, out, error);
  }
  return cudaGetLastError();
}

}  // namespace mpsb
