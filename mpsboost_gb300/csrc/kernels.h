// Launch interface of the sm_103a kernels (host and device code include this).
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "device.cuh"

namespace mpsb {

// Device pointers and sizes of one training session, passed by value to every kernel.
struct TrainerDev {
  // dataset
  const uint8_t* bins;          // u8 bins for histograms: row r, feature f at
                                //   r * bins_row_stride + (f/32) * bins_block_stride + f%32
  uint64_t bins_row_stride, bins_block_stride;
  const uint8_t* bins_fm;       // [features][n_rows] feature-major u8 bins (routing rows)
  const uint32_t* bin_count;    // [features]
  const uint8_t* has_missing;   // [features]
  // Histogram slots per feature: 256 (u8 bins, missing rows at slot 255), or for wide
  // datasets (a feature with more than 256 bins, or 256 bins and missing values) a larger
  // multiple of 256 with missing rows at slot slots - 1; wide datasets keep u16 copies of
  // the bins in place of the u8 ones.
  uint32_t slots = kSlots;
  const uint16_t* bins16;       // wide: [nfb][n_rows][32] column blocks (else null)
  const uint16_t* bins16_fm;    // wide: [features][n_rows] (else null)
  uint32_t n_rows, features, nfb, n_trees;
  // per-tree arrays
  const double* labels;         // [n_rows]
  const double* weights;        // [n_rows], [n_trees][n_rows] or null (unit weights)
  uint32_t weights_per_tree;
  uint32_t objective;
  double* preds;                // [n_trees][n_rows]
  float2* gh;                   // gh_ordered: [n_trees][2][seg_stride] in row-segment order
                                // (moved along by the partition); else [n_trees][n_rows]
  uint32_t gh_ordered;
  uint32_t* rows;               // [n_trees][2][seg_stride] row ids of the level's segments
  uint32_t seg_stride;          // positions per (tree, parity) of rows / gh: n_rows, or the
                                // largest sample of a forest (a row appears once per draw)
  // Forest samples (null for boosting): per tree the multiset of rows it trains on,
  // [n_trees][seg_stride] in ascending row order, and its size; the feature rank of each
  // feature in the tree's subset (random thresholds hash the rank) and per-tree seeds.
  const uint32_t* sample_rows;
  const uint32_t* sample_count;   // [n_trees]
  const uint32_t* feature_rank;   // [n_trees][features] or null (rank = feature)
  const uint32_t* tree_seeds;     // [n_trees] or null (params.random_seed)
  uint32_t skip_apply;            // 1: no prediction update (forest trees are single-round)
  uint32_t unit_hess;             // every row's hessian is 1 (no weights; squared error or
                                  // quantile): fixed-point builds take kModeFixedCG
  TreeState* trees;             // [n_trees]
  TreeParams params;
  const int8_t* monotonic;      // [features] or null
  const uint32_t* group_masks;  // [n_groups][path_words]
  const uint32_t* tree_feature_masks;  // [n_trees][path_words] or null
  // histogram slots: [n_slots][features][slots] x {count, g, h} 64-bit words
  unsigned long long* hist;
  uint32_t* free_stack;         // [n_slots]
  uint32_t n_slots;
  // level buffers (index = level parity)
  NodeRec* nodes[2];            // [max_level_nodes]
  uint32_t* node_path[2];       // [max_level_nodes][path_words]
  uint32_t* node_allowed[2];    // [max_level_nodes][path_words]
  uint32_t max_level_nodes;
  SplitRec* partial;            // [max_level_nodes][n_fchunks]
  // Two-phase split scan (scan_two_phase: the FP32 screen applies): [max_level_nodes]
  // maximum FP32 screen score of each node's certainly admissible candidates (float
  // bits; zeroed by each level's zero_build_slots_kernel, which every scan of the trainer
  // follows) and [max_level_nodes][n_fchunks] each chunk's maximum
  // and exact flag. Null node_screen: one launch, each feature screened on its own (the
  // per-feature entry point needs every feature's best split).
  uint32_t* node_screen;
  uint32_t* chunk_screen;
  uint32_t scan_two_phase;
  uint32_t n_fchunks;           // feature chunks of the split scan (32 features each)
  BuildEntry* build;            // [max_level_nodes]
  uint32_t* build_prefix;       // [max_level_nodes + 1] chunk prefix
  SubEntry* sub;                // [max_level_nodes]
  PartEntry* part;              // [max_level_nodes]
  uint32_t* part_prefix;        // [max_level_nodes + 1] chunk prefix
  uint32_t* part_counts;        // [max_part_chunks] left rows per chunk
  uint32_t* part_offsets;       // [max_part_chunks] left rows before the chunk in its node
  uint32_t* part_flags;         // [max_part_chunks][kPartChunk / 32]
  uint32_t max_part_chunks;
  LeafSeg* leafseg;             // [max_leafsegs]
  uint32_t* leaf_of;            // [n_trees][n_rows]: 2 x leaf segment + side, per row of the
                                // round (kNoLeaf between rounds)
  double* leaf_steps;           // [2 * max_leafsegs]: lr x leaf value per (segment, side)
  uint32_t* leaf_prefix;        // [max_leafsegs + 1]
  uint32_t max_leafsegs;
  TreeNodeOut* tree_nodes;      // [n_trees][max_tree_nodes]
  uint32_t max_tree_nodes;
  Control* ctl;
  uint32_t item_rows;           // rows per histogram work item (<= kItemRowsMax); 0: the
                                // level's adaptive value ctl->item_rows
  uint32_t sm_count;
  uint32_t items_per_sm;        // histogram work items per SM of the adaptive item size (0: 3)
  uint32_t mode;                // kModeFixed / kModeFloat
  uint32_t ovr;                 // labels are class ids; tree t fits class t (logistic)
  uint32_t n_classes;           // native softmax: K classes, one tree per class in turn;
                                // preds holds the margins [K][n_rows] and the round
                                // counter modulo K is the class of the current tree
  uint32_t scan_threads;        // block size of the split scan (multiple of 32)
  uint32_t fused_sub;           // level-wise siblings are subtracted by the split scan
                                // (NodeRec::sub_from), not by subtract_kernel
  // finalize scratch
  uint32_t* scratch_flags;      // [max_level_nodes]
  uint32_t* scratch_prefix;     // [max_level_nodes] valid-prefix, then accepted-prefix
  uint32_t* scratch_aux;        // [max_level_nodes] free-slot prefix
  uint32_t* tree_scratch;       // [n_trees][4]
  // model output: per round, per tree, max_tree_nodes nodes + node counts
  TreeNodeOut* model_nodes;     // [max_rounds][n_trees][max_tree_nodes]
  uint32_t* model_counts;       // [max_rounds][n_trees]
  uint32_t* round_counter;      // rounds completed (device)
  uint32_t max_rounds;
  // Histogram item range of one launch: [item_begin, item_end); item_end 0 = the whole
  // level (ctl->hist_items). Per-node launches of the plain path set a node's range.
  uint32_t item_begin, item_end;
  // Leaf-wise growth (growth_strategy 1; null for level-wise): per tree the active leaves
  // with their interaction path and allowed-feature words, the active count, a done flag,
  // and a private stack of histogram slots; the scanned children of a step map to
  // (tree << 16 | active index).
  LeafActive* lw_active;        // [n_trees][lw_cap]
  uint32_t* lw_path;            // [n_trees][lw_cap][path_words]
  uint32_t* lw_allowed;         // [n_trees][lw_cap][path_words]
  uint32_t* lw_count;           // [n_trees]
  uint32_t* lw_done;            // [n_trees]
  uint32_t* lw_slots;           // [n_trees][lw_slot_cap] free slots
  uint32_t* lw_slot_top;        // [n_trees]
  uint32_t* lw_scan_map;        // [2 * n_trees]
  uint32_t lw_cap, lw_slot_cap, lw_max_active, lw_max_leaves;
  // Root count/hessian histograms of the fit's first round: [n_trees][features][slots]
  // {count, qh} and the hessian scale they were built with (null: not reused).
  unsigned long long* root_cache;
  int* root_cache_kh;
};

struct HistConfig {
  int threads = 768;        // fixed and float builds
  int stages = 2;
  int root_threads = 1024;  // gradient-only root builds (64 KB histogram)
  // Register-direct fixed-point builds (hist_build_direct_kernel: each lane loads a whole
  // row's 32-byte feature block, no shared-memory staging; flush by TMA bulk reductions);
  // threads 512 or 768. The opt-in TMA staging (bins_tmap) takes precedence. The trainer
  // turns it on; the node-level entries keep the staged kernel.
  bool direct = false;
  // Wide datasets (more than 256 slots per feature): threads of hist_build_wide_kernel,
  // 1024 (32 warps hide the gathers' latency: 1.3x faster than 512 at 512 and 1024 bins
  // on 4M x 128) or 512.
  int wide_threads = 1024;
  // Tensor map of the row-major bins ({row stride, n_rows} u8, box 32 x 1): row-major
  // fixed-point builds stage gathered rows with TMA gather4 copies (opt-in). Null: cp.async.
  const CUtensorMap* bins_tmap = nullptr;
};

// Encodes the tensor map of a row-major bins matrix (rows x row_stride bytes). Returns
// false where the CUDA driver offers no tensor maps.
bool encode_bins_tmap(CUtensorMap* map, const uint8_t* bins, uint64_t row_stride, uint32_t n_rows);

cudaError_t launch_hist_build(const TrainerDev& a, const HistConfig& cfg, int grid,
                              cudaStream_t stream);
cudaError_t launch_fill_f64(double* dst, uint64_t n, double value, cudaStream_t stream);
cudaError_t launch_round_begin(const TrainerDev& a, cudaStream_t stream);
cudaError_t launch_gradients(const TrainerDev& a, int grid, cudaStream_t stream);
cudaError_t launch_round_setup(const TrainerDev& a, cudaStream_t stream);
cudaError_t launch_zero_build_slots(const TrainerDev& a, int grid, cudaStream_t stream);
cudaError_t launch_root_stats(const TrainerDev& a, cudaStream_t stream);
// Leaf-wise growth: after the root's split scan (init), per step (select before the
// partition / histogram / subtraction / split scan of the chosen leaves' children, merge
// after), and the leaf segments at the end (finish).
cudaError_t launch_leafwise_init(const TrainerDev& a, cudaStream_t stream);
cudaError_t launch_leafwise_select(const TrainerDev& a, cudaStream_t stream);
cudaError_t launch_leafwise_merge(const TrainerDev& a, cudaStream_t stream);
cudaError_t launch_leafwise_finish(const TrainerDev& a, cudaStream_t stream);
// save != 0: copy the roots' count and hessian words into root_cache; else restore them
// into the roots' slots (after a gradient-only build).
cudaError_t launch_root_cache(const TrainerDev& a, int save, int grid, cudaStream_t stream);
cudaError_t launch_subtract(const TrainerDev& a, int grid, cudaStream_t stream);
cudaError_t launch_split_scan(const TrainerDev& a, int parity, int grid, cudaStream_t stream);
uint32_t split_scan_kernels(const TrainerDev& a);  // launches per launch_split_scan
cudaError_t launch_finalize(const TrainerDev& a, int parity, uint32_t depth, cudaStream_t stream);
cudaError_t launch_partition(const TrainerDev& a, int grid, cudaStream_t stream);
cudaError_t launch_partition_count(const TrainerDev& a, int grid, cudaStream_t stream);
cudaError_t launch_partition_finish(const TrainerDev& a, int grid, cudaStream_t stream);
cudaError_t launch_apply_leaves(const TrainerDev& a, int grid, cudaStream_t stream);
cudaError_t launch_round_end(const TrainerDev& a, cudaStream_t stream);
cudaError_t launch_squared_error(const double* labels, const double* preds, uint64_t n,
                                 double* out_pairs, uint32_t* error, cudaStream_t stream);
// Bins from the u8 feature-major copy (missing rows at 255), or with bins16_fm set from
// the u16 one (missing rows at slots - 1).
cudaError_t launch_predict(const uint8_t* bins_fm, const uint16_t* bins16_fm, uint32_t slots,
                           uint32_t n_rows, uint32_t nfb, const uint8_t* has_missing,
                           const TreeNodeOut* nodes, const uint32_t* tree_offsets,
                           uint32_t n_trees, double base, double learning_rate, double* out,
                           uint32_t* error, cudaStream_t stream);
// Wide datasets: one feature block fb of the u16 copies ([nfb][n_rows][32] column blocks
// and [features][n_rows]) from a staged copy of its source features, missing rows at
// slots - 1.
cudaError_t launch_pack_bins16_block(const void* src_block, uint32_t width,
                                     const uint8_t* missing_block, const uint32_t* bin_count,
                                     uint32_t n_rows, uint32_t features, uint32_t fb,
                                     uint32_t slots, uint16_t* out_blocked, uint16_t* out_fm,
                                     uint32_t* error, cudaStream_t stream);
// One feature block fb of the dataset from a staged copy of its source features
// (src_block / missing_block start at feature 32 * fb).
cudaError_t launch_pack_bins_block(const void* src_block, uint32_t width, const uint8_t* missing_block,
                                   const uint32_t* bin_count, uint32_t n_rows, uint32_t features,
                                   uint32_t nfb, uint32_t fb, uint8_t* out_rows, uint8_t* out_blocked,
                                   uint8_t* out_fm, uint32_t* error, cudaStream_t stream);
cudaError_t launch_pack_bins(const void* src, uint32_t width, const uint8_t* missing,
                             const uint32_t* bin_count, uint32_t n_rows, uint32_t features,
                             uint32_t nfb, uint8_t* out_rows, uint8_t* out_blocked,
                             uint8_t* out_fm, uint32_t* error, cudaStream_t stream);
// Raises `kernel`'s dynamic shared memory limit to `bytes` on the current device before
// its first launch there. The limit is an attribute of the function in that device's
// context, so it is set once per device: bit d of `devices` records device d (devices
// past 63 set it before every launch). Two host threads that race past the check both set
// the same value, which is harmless.
template <typename Kernel>
inline cudaError_t opt_in_dynamic_smem(std::atomic<unsigned long long>& devices, Kernel kernel,
                                       size_t bytes) {
  int device = 0;
  cudaError_t err = cudaGetDevice(&device);
  if (err != cudaSuccess) return err;
  const unsigned long long bit = device >= 0 && device < 64 ? 1ull << device : 0ull;
  if (bit && (devices.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (err == cudaSuccess && bit) devices.fetch_or(bit, std::memory_order_acq_rel);
  return err;
}

// Number of kernels each launch_* helper enqueues (launch accounting).
constexpr int kPartitionKernels = 3;

}  // namespace mpsb
