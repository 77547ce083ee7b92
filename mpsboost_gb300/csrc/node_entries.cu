// Node-level entries of the backend contract (include/mpsboost/backend.hpp:52-135 and the
// MPS test hooks 164-185), run on the same sm_103a kernels as the training session:
//   mpsb_cuda_squared_error           GradientComputer::ComputeSquaredError
//   mpsb_cuda_build_histograms        HistogramBuilder::BuildHistograms
//   mpsb_cuda_build_layer_histograms  LayerHistogramBuilder::BuildLayerHistograms
//   mpsb_cuda_scan_splits             ScanSplitsForTest, with FindBestSplit semantics
//   mpsb_cuda_partition_rows          PartitionRowsForTest, missing rows by default_left
// Each call uploads its borrowed host inputs, runs, copies the result back and keeps no
// pointer to them (backend.hpp:68-70).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "host_types.h"

using namespace mpsb;

namespace {

// Device buffers and kernel arguments of one node-level call.
struct Session {
  std::vector<std::unique_ptr<DevBuf>> bufs;
  TrainerDev a{};
  template <class T>
  T* alloc(size_t count) {
    bufs.emplace_back(new DevBuf);
    bufs.back()->alloc(count * sizeof(T));
    return bufs.back()->as<T>();
  }
  template <class T>
  T* upload(const T* host, size_t count, cudaStream_t s) {
    T* d = alloc<T>(count);
    if (count) CK(cudaMemcpyAsync(d, host, count * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
  }
};

void base_session(Session& ss, mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds) {
  dataset_ready(ds);
  TrainerDev& a = ss.a;
  a.bins = ds->bins.as<uint8_t>();
  a.bins_row_stride = uint64_t(ds->nfb) * kBlockFeatures;
  a.bins_block_stride = kBlockFeatures;
  a.bins_fm = ds->bins_fm.as<uint8_t>();
  a.slots = ds->slots;
  a.bins16 = ds->bins16.as<uint16_t>();
  a.bins16_fm = ds->bins16_fm.as<uint16_t>();
  a.sm_count = uint32_t(b->sm_count);
  a.bin_count = ds->bin_count.as<uint32_t>();
  a.has_missing = ds->has_missing.as<uint8_t>();
  a.n_rows = ds->n_rows;
  a.seg_stride = ds->n_rows;  // the partition entry writes parity 1 at this offset
  a.features = ds->features;
  a.nfb = ds->nfb;
  a.n_trees = 1;
  a.mode = b->hist_mode == MPSB_HIST_FLOAT ? kModeFloat : kModeFixed;
  a.ctl = ss.alloc<Control>(1);
  CK(cudaMemsetAsync(a.ctl, 0, sizeof(Control), b->stream));
}

std::vector<uint32_t> rows_u32(const uint64_t* rows, uint64_t n, uint32_t n_rows,
                               const char* what) {
  std::vector<uint32_t> out(n);
  for (uint64_t i = 0; i < n; ++i) {
    if (rows[i] >= n_rows) throw TrainingError(what);
    out[i] = uint32_t(rows[i]);
  }
  return out;
}

// FP64 pairs -> FP32 pairs (the device representation), with the checks of
// reference_backend.cpp:46-50.
std::vector<float> pairs32(const double* pairs, uint64_t n) {
  std::vector<float> out(2 * n);
  for (uint64_t i = 0; i < n; ++i) {
    const double g = pairs[2 * i], h = pairs[2 * i + 1];
    if (!std::isfinite(g) || !std::isfinite(h) || h < 0.0)
      throw TrainingError("Gradient/Hessian must be finite and Hessian non-negative");
    out[2 * i] = float(g);
    out[2 * i + 1] = float(h);
    if (!std::isfinite(out[2 * i]) || !std::isfinite(out[2 * i + 1]))
      throw TrainingError("Gradient/Hessian exceed the float32 range of the device path");
  }
  return out;
}

// Build the histograms of n_nodes row sets (concatenated rows, node_offsets) into slots
// 0..n_nodes-1. Returns the session (slots stay on the device) and the tree state.
void build_slots(Session& ss, mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                 const uint64_t* rows, const uint64_t* offsets, uint32_t n_nodes,
                 const double* pairs, uint64_t n_pairs, TreeState* state_out) {
  cudaStream_t s = b->stream;
  if (n_pairs != ds->n_rows)
    throw TrainingError("Gradient count does not match binned dataset row count");
  for (uint32_t i = 0; i < n_nodes; ++i)
    if (offsets[i + 1] <= offsets[i]) throw TrainingError("Node row set must not be empty");
  const uint64_t total = offsets[n_nodes];
  if (total >= 0xFFFFFFFFull) throw UnsupportedError("too many rows in one call");
  base_session(ss, b, ds);
  TrainerDev& a = ss.a;
  const std::vector<uint32_t> r32 = rows_u32(rows, total, ds->n_rows, "Histogram row index is out of bounds");
  const std::vector<float> p32 = pairs32(pairs, n_pairs);
  a.rows = ss.upload(r32.data(), r32.size(), s);
  a.gh = reinterpret_cast<float2*>(ss.upload(p32.data(), p32.size(), s));
  TreeState st{};
  fixed_scales(p32.data(), n_pairs, ds->n_rows, &st.kg, &st.kh);
  st.inv_g = std::ldexp(1.0, -st.kg);
  st.inv_h = std::ldexp(1.0, -st.kh);
  a.trees = ss.upload(&st, 1, s);
  *state_out = st;
  // rows per work item: spread the call over the SMs, within the packing bound
  const uint64_t target = uint64_t(b->sm_count) * 4;
  uint64_t per = (total * ds->nfb + target - 1) / target;
  per = std::min<uint64_t>(std::max<uint64_t>((per + 511) / 512 * 512, 512), kItemRowsMax);
  a.item_rows = uint32_t(per);
  std::vector<BuildEntry> build(n_nodes);
  std::vector<uint32_t> prefix(n_nodes + 1, 0);
  for (uint32_t i = 0; i < n_nodes; ++i) {
    const uint64_t cnt = offsets[i + 1] - offsets[i];
    build[i] = BuildEntry{0, 0, uint32_t(offsets[i]), uint32_t(cnt), i, 0};
    prefix[i + 1] = prefix[i] + uint32_t((cnt + a.item_rows - 1) / a.item_rows);
  }
  a.build = ss.upload(build.data(), build.size(), s);
  a.build_prefix = ss.upload(prefix.data(), prefix.size(), s);
  a.n_slots = n_nodes;
  a.hist = ss.alloc<unsigned long long>(size_t(n_nodes) * ds->features * ds->slots * 3);
  Control c{};
  c.n_build = n_nodes;
  c.hist_items = prefix[n_nodes] * ds->nfb;
  CK(cudaMemcpyAsync(a.ctl, &c, sizeof c, cudaMemcpyHostToDevice, s));
  CK(launch_zero_build_slots(a, b->sm_count * 8, s));
  CK(launch_hist_build(a, HistConfig{}, b->sm_count, s));
}

void check_ctl(const TrainerDev& a, cudaStream_t s) {
  Control c;
  CK(cudaMemcpyAsync(&c, a.ctl, sizeof c, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (c.error) throw TrainingError(describe_device_error(c.error));
}

// Slots -> features x bin_count HistogramBins, missing rows folded into bin 0 as in the
// reference dataset (binned_dataset.cpp:169-176).
void decode_slots(const mpsb_cuda_dataset* ds, const std::vector<unsigned long long>& slots,
                  uint32_t n_nodes, int mode, const TreeState& st, mpsb_histogram_bin* out) {
  const uint32_t F = ds->features;
  const size_t miss = ds->slots - 1;  // missing rows' slot
  size_t k = 0;
  for (uint32_t i = 0; i < n_nodes; ++i) {
    for (uint32_t f = 0; f < F; ++f) {
      const unsigned long long* base = slots.data() + (size_t(i) * F + f) * ds->slots * 3;
      const bool hm = ds->h_has_missing[f] != 0;
      for (uint32_t bin = 0; bin < ds->h_bin_count[f]; ++bin) {
        unsigned long long cnt = base[bin * 3];
        mpsb_histogram_bin o{};
        if (mode == kModeFixed) {
          long long qg = (long long)base[bin * 3 + 1], qh = (long long)base[bin * 3 + 2];
          if (bin == 0 && hm) {
            cnt += base[miss * 3];
            qg += (long long)base[miss * 3 + 1];
            qh += (long long)base[miss * 3 + 2];
          }
          o.gradient_sum = double(qg) * st.inv_g;
          o.hessian_sum = double(qh) * st.inv_h;
        } else {
          double g, h;
          std::memcpy(&g, &base[bin * 3 + 1], 8);
          std::memcpy(&h, &base[bin * 3 + 2], 8);
          if (bin == 0 && hm) {
            double mg, mh;
            std::memcpy(&mg, &base[miss * 3 + 1], 8);
            std::memcpy(&mh, &base[miss * 3 + 2], 8);
            cnt += base[miss * 3];
            g += mg;
            h += mh;
          }
          o.gradient_sum = g;
          o.hessian_sum = h;
        }
        o.count = cnt;
        out[k++] = o;
      }
    }
  }
}

}  // namespace

extern "C" {

int mpsb_cuda_squared_error(mpsb_cuda_backend* b, const double* labels, const double* preds,
                            uint64_t n, double* out) {
  return guard([&] {
    if (n == 0) throw TrainingError("Labels must not be empty");
    b->activate();
    Session ss;
    cudaStream_t s = b->stream;
    const double* dl = ss.upload(labels, n, s);
    const double* dp = ss.upload(preds, n, s);
    double* d_out = ss.alloc<double>(2 * n);
    CK(launch_squared_error(dl, dp, n, d_out, b->error.as<uint32_t>(), s));
    CK(cudaMemcpyAsync(out, d_out, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (b->take_error()) throw TrainingError("label and prediction must be finite");
  });
}

int mpsb_cuda_build_layer_histograms(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                                     const uint64_t* rows, const uint64_t* node_offsets,
                                     uint32_t n_nodes, const double* pairs, uint64_t n_pairs,
                                     mpsb_histogram_bin* out) {
  return guard([&] {
    if (n_nodes == 0) return;
    b->activate();
    Session ss;
    TreeState st;
    build_slots(ss, b, ds, rows, node_offsets, n_nodes, pairs, n_pairs, &st);
    check_ctl(ss.a, b->stream);
    std::vector<unsigned long long> slots(size_t(n_nodes) * ds->features * ds->slots * 3);
    CK(cudaMemcpy(slots.data(), ss.a.hist, slots.size() * 8, cudaMemcpyDeviceToHost));
    decode_slots(ds, slots, n_nodes, int(ss.a.mode), st, out);
  });
}

int mpsb_cuda_build_histograms(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                               const uint64_t* rows, uint64_t n_rows, const double* pairs,
                               uint64_t n_pairs, mpsb_histogram_bin* out) {
  const uint64_t offsets[2] = {0, n_rows};
  return mpsb_cuda_build_layer_histograms(b, ds, rows, offsets, 1, pairs, n_pairs, out);
}

int mpsb_cuda_scan_splits(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                          const uint64_t* rows, uint64_t n_rows, const double* pairs,
                          uint64_t n_pairs, const mpsb_train_params* p,
                          mpsb_split_candidate* out) {
  return guard([&] {
    if (n_rows == 0) throw TrainingError("Split-scan row set must not be empty");
    validate_tree_params(*p, ds->features);
    b->activate();
    cudaStream_t s = b->stream;
    Session ss;
    TreeState st;
    const uint64_t offsets[2] = {0, n_rows};
    build_slots(ss, b, ds, rows, offsets, 1, pairs, n_pairs, &st);
    TrainerDev& a = ss.a;
    const uint32_t F = ds->features, W = (F + 31) / 32;
    TreeParams& tp = a.params;
    tp.min_samples_leaf = p->min_samples_leaf;
    tp.min_child_weight = p->min_child_weight;
    tp.reg_lambda = p->reg_lambda;
    tp.reg_alpha = p->reg_alpha;
    tp.max_delta_step = p->max_delta_step;
    tp.gamma = p->gamma;
    tp.min_gain_to_split = p->min_gain_to_split;
    tp.learning_rate = p->learning_rate;
    tp.max_depth = p->max_depth;
    tp.split_strategy = p->split_strategy;
    tp.random_seed = p->random_seed;
    tp.has_monotonic = p->n_monotonic ? 1 : 0;
    tp.path_words = W;
    set_screen_constants(tp);
    if (p->n_monotonic) a.monotonic = ss.upload(p->monotonic_constraints, F, s);
    NodeRec node{};
    node.seg_off = 0;
    node.seg_cnt = uint32_t(n_rows);
    node.lo = -INFINITY;
    node.hi = INFINITY;
    a.nodes[0] = ss.upload(&node, 1, s);
    std::vector<uint32_t> ones(W, 0xffffffffu);
    a.node_allowed[0] = ss.upload(ones.data(), W, s);
    a.tree_nodes = ss.alloc<TreeNodeOut>(1);
    a.max_tree_nodes = 1;
    a.scan_threads = 32;  // one feature per CTA: partial[f] is feature f's best split
    a.n_fchunks = F;
    a.partial = ss.alloc<SplitRec>(F);
    CK(launch_root_stats(a, s));
    const uint32_t one = 1;
    CK(cudaMemcpyAsync(&a.ctl->n_nodes, &one, sizeof one, cudaMemcpyHostToDevice, s));
    CK(launch_split_scan(a, 0, b->sm_count * 8, s));
    check_ctl(a, s);
    std::vector<SplitRec> rec(F);
    CK(cudaMemcpy(rec.data(), a.partial, F * sizeof(SplitRec), cudaMemcpyDeviceToHost));
    for (uint32_t f = 0; f < F; ++f) {
      mpsb_split_candidate& o = out[f];
      std::memset(&o, 0, sizeof o);
      o.valid = rec[f].valid;
      o.feature = f;
      if (!rec[f].valid) continue;
      o.threshold_bin = rec[f].threshold;
      o.default_left = rec[f].default_left;
      o.left_count = rec[f].lcount;
      o.right_count = rec[f].rcount;
      o.left_gradient_sum = rec[f].lg;
      o.left_hessian_sum = rec[f].lh;
      o.right_gradient_sum = rec[f].rg;
      o.right_hessian_sum = rec[f].rh;
      o.gain = rec[f].gain;
    }
  });
}

int mpsb_cuda_partition_rows(mpsb_cuda_backend* b, const mpsb_cuda_dataset* ds,
                             const uint64_t* rows, uint64_t n_rows, uint32_t feature,
                             uint32_t threshold_bin, int default_left, uint64_t* left_out,
                             uint64_t* right_out, uint64_t* n_left) {
  return guard([&] {
    if (n_rows == 0) throw TrainingError("Partition row set must not be empty");
    if (feature >= ds->features || threshold_bin >= ds->h_bin_count[feature])
      throw TrainingError("Partition feature or threshold is out of bounds");
    if (n_rows >= 0xFFFFFFFFull - ds->n_rows) throw UnsupportedError("too many rows in one call");
    b->activate();
    cudaStream_t s = b->stream;
    Session ss;
    base_session(ss, b, ds);
    TrainerDev& a = ss.a;
    const std::vector<uint32_t> r32 = rows_u32(rows, n_rows, ds->n_rows, "Partition row index is out of bounds");
    // Input rows at [0, n_rows); the scatter writes the other parity at n_rows_dataset.
    a.rows = ss.alloc<uint32_t>(size_t(ds->n_rows) + n_rows);
    CK(cudaMemcpyAsync(a.rows, r32.data(), n_rows * 4, cudaMemcpyHostToDevice, s));
    const uint32_t chunks = uint32_t((n_rows + kPartChunk - 1) / kPartChunk);
    PartEntry pe{0, 0, 0, uint32_t(n_rows), feature, threshold_bin, default_left ? 1u : 0u, 0};
    a.part = ss.upload(&pe, 1, s);
    const uint32_t prefix[2] = {0, chunks};
    a.part_prefix = ss.upload(prefix, 2, s);
    a.part_counts = ss.alloc<uint32_t>(chunks);
    a.part_offsets = ss.alloc<uint32_t>(chunks);
    a.part_flags = ss.alloc<uint32_t>(size_t(chunks) * (kPartChunk / 32));
    a.max_part_chunks = chunks;
    Control c{};
    c.n_part = 1;
    c.part_chunks = chunks;
    CK(cudaMemcpyAsync(a.ctl, &c, sizeof c, cudaMemcpyHostToDevice, s));
    CK(launch_partition_count(a, b->sm_count * 4, s));
    std::vector<uint32_t> counts(chunks);
    CK(cudaMemcpyAsync(counts.data(), a.part_counts, chunks * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    uint64_t nl = 0;
    for (uint32_t v : counts) nl += v;
    pe.lcount = uint32_t(nl);
    CK(cudaMemcpyAsync(a.part, &pe, sizeof pe, cudaMemcpyHostToDevice, s));
    CK(launch_partition_finish(a, b->sm_count * 4, s));
    check_ctl(a, s);
    std::vector<uint32_t> res(n_rows);
    CK(cudaMemcpy(res.data(), a.rows + ds->n_rows, n_rows * 4, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < nl; ++i) left_out[i] = res[i];
    for (uint64_t i = nl; i < n_rows; ++i) right_out[i - nl] = res[i];
    *n_left = nl;
  });
}

}  // extern "C"
