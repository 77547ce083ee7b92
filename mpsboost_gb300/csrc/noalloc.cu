// Histogram build for callers that cannot allocate device memory.
//
// Some callers of this library are not allowed to call cudaMalloc: a plugin running
// inside a host process whose device memory is owned by that process's own pool
// allocator (a stray cudaMalloc would bypass its accounting and can fail once the pool
// has reserved the GPU), or a latency-bound serving loop where cudaMalloc's implicit
// device synchronisation is not acceptable. They already hold their inputs and outputs
// in device memory. mpsb_cuda_build_histogram_noalloc builds one node's fixed-point
// histogram from those caller-owned buffers and keeps every intermediate (the int64
// accumulation slot, the work table, the control block, the scale words) in the
// file-scope array below, so it calls no allocating routine at all.
//
// The array is a fixed kNoAllocScratchBytes (2 MiB) of device memory that every GPU
// loading this library keeps until the process exits. Its device address is looked up
// with cudaGetSymbolAddress on the first call on each device, with that device current;
// make that first call before any stream capture. Every call shares the array and the
// array keeps the last call's contents, so each call clears what must start at zero, and
// calls whose work overlaps on the GPU (different streams, or different host threads on
// the same device) race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "host_types.h"

using namespace mpsb;

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(2) << 20;
constexpr uint32_t kNoAllocMaxFeatures = 256;

// Scratch layout (byte offsets). The slot comes last: features x 256 x 3 words.
constexpr size_t kCtlOff = 0;        // Control
constexpr size_t kTreeOff = 256;     // TreeState (+ the scale maxima)
constexpr size_t kBuildOff = 512;    // BuildEntry[1]
constexpr size_t kPrefixOff = 768;   // uint32 prefix[2]
constexpr size_t kSlotOff = 1024;
static_assert(sizeof(Control) <= 256 && sizeof(TreeState) <= 256 && sizeof(BuildEntry) <= 256,
              "scratch header layout");
static_assert(kSlotOff + size_t(kNoAllocMaxFeatures) * kSlots * 3 * 8 <= kNoAllocScratchBytes,
              "scratch holds the largest slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct DeviceScratch {
  void* ptr = nullptr;
  int sm_count = 0;
};
std::mutex g_scratch_mutex;
DeviceScratch g_scratch[64];

// Device address of the scratch array on the current device (looked up once per device).
DeviceScratch scratch_for_current_device() {
  int device = 0;
  CK(cudaGetDevice(&device));
  if (device < 0 || device >= 64) throw UnsupportedError("device index beyond 63");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  DeviceScratch& s = g_scratch[device];
  if (s.ptr == nullptr) {
    void* ptr = nullptr;
    CK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    s.ptr = ptr;
    s.sm_count = sms;
  }
  return s;
}

// max |g| and max h over all dataset rows (the same scale rule as every other entry).
// A pair that is not finite, or a negative hessian, sets ctl->error: the entry cannot
// raise an error without synchronising, so the histogram is then skipped and every bin
// comes back with NaN sums.
__global__ void noalloc_maxima_kernel(const float2* pairs, uint32_t n, TreeState* st, Control* ctl) {
  uint32_t mg = 0, mh = 0;
  bool bad = false;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 p = pairs[i];
    bad |= !isfinite(p.x) || !isfinite(p.y) || p.y < 0.0f;
    mg = max(mg, __float_as_uint(fabsf(p.x)));
    mh = max(mh, __float_as_uint(fmaxf(p.y, 0.0f)));
  }
  for (int off = 16; off > 0; off >>= 1) {
    mg = max(mg, __shfl_xor_sync(0xffffffffu, mg, off));
    mh = max(mh, __shfl_xor_sync(0xffffffffu, mh, off));
  }
  bad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&st->max_abs_g_bits, mg);
    atomicMax(&st->max_h_bits, mh);
    if (bad) atomicOr(&ctl->error, 1u);
  }
}

__global__ void noalloc_setup_kernel(TreeState* st, BuildEntry* build, uint32_t* prefix,
                                     Control* ctl, uint32_t n_rows, uint32_t item_rows,
                                     uint32_t nfb) {
  const float mg = __uint_as_float(st->max_abs_g_bits), mh = __uint_as_float(st->max_h_bits);
  int e;
  frexpf(mg, &e);
  st->kg = mg > 0.0f ? 30 - e : 0;
  frexpf(mh, &e);
  st->kh = mh > 0.0f ? 30 - e : 0;
  st->inv_g = ldexp(1.0, -st->kg);
  st->inv_h = ldexp(1.0, -st->kh);
  BuildEntry b;
  b.tree = 0;
  b.parity = 0;
  b.seg_off = 0;
  b.seg_cnt = n_rows;
  b.slot = 0;
  b.pad = 0;
  *build = b;
  const uint32_t chunks = (n_rows + item_rows - 1) / item_rows;
  prefix[0] = 0;
  prefix[1] = chunks;
  ctl->n_build = 1;
  ctl->hist_items = ctl->error ? 0u : chunks * nfb;  // invalid pairs: no histogram work
  ctl->hist_counter = 0;
}

// Slot (int64 fixed point) -> [features][256] {count, FP64 G, FP64 H}.
// Invalid pairs (ctl->error): count 0 and NaN sums in every bin.
__global__ void noalloc_decode_kernel(const unsigned long long* slot, const TreeState* st,
                                      const Control* ctl, uint32_t cells, mpsb_histogram_bin* out) {
  const bool bad = ctl->error != 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cells; i += gridDim.x * blockDim.x) {
    mpsb_histogram_bin o;
    o.count = bad ? 0ull : slot[3 * size_t(i)];
    o.gradient_sum = bad ? __longlong_as_double(0x7FF8000000000000ll)
                         : q_image((long long)slot[3 * size_t(i) + 1], st->inv_g);
    o.hessian_sum = bad ? __longlong_as_double(0x7FF8000000000000ll)
                        : q_image((long long)slot[3 * size_t(i) + 2], st->inv_h);
    out[i] = o;
  }
}

}  // namespace

extern "C" int mpsb_cuda_build_histogram_noalloc(const uint8_t* bins, uint32_t dataset_rows,
                                                  uint32_t features, const uint32_t* rows,
                                                  uint32_t n_rows, const float* pairs,
                                                  mpsb_histogram_bin* out, void* stream) {
  return guard([&] {
    if (!bins || !rows || !pairs || !out) throw TrainingError("null device pointer");
    if (features == 0 || dataset_rows == 0) throw DataError("dataset must contain at least one row and one feature");
    if (features > kNoAllocMaxFeatures)
      throw UnsupportedError("mpsb_cuda_build_histogram_noalloc supports at most " +
                             std::to_string(kNoAllocMaxFeatures) + " features (its fixed 2 MiB scratch)");
    if (n_rows == 0) throw TrainingError("Node row set must not be empty");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const DeviceScratch sc = scratch_for_current_device();
    unsigned char* base = static_cast<unsigned char*>(sc.ptr);
    Control* ctl = reinterpret_cast<Control*>(base + kCtlOff);
    TreeState* st = reinterpret_cast<TreeState*>(base + kTreeOff);
    BuildEntry* build = reinterpret_cast<BuildEntry*>(base + kBuildOff);
    uint32_t* prefix = reinterpret_cast<uint32_t*>(base + kPrefixOff);
    unsigned long long* slot = reinterpret_cast<unsigned long long*>(base + kSlotOff);
    const uint32_t nfb = (features + kBlockFeatures - 1) / kBlockFeatures;
    const size_t slot_bytes = size_t(features) * kSlots * 3 * 8;
    // Clear what the previous call left: header words, maxima and the accumulation slot.
    CK(cudaMemsetAsync(base, 0, kSlotOff, s));
    CK(cudaMemsetAsync(slot, 0, slot_bytes, s));
    const float2* gh = reinterpret_cast<const float2*>(pairs);
    const int grid = sc.sm_count * 4;
    noalloc_maxima_kernel<<<grid, 256, 0, s>>>(gh, dataset_rows, st, ctl);
    CK(cudaGetLastError());
    const uint64_t target = uint64_t(sc.sm_count) * 4;
    uint64_t per = (uint64_t(n_rows) * nfb + target - 1) / target;
    per = std::min<uint64_t>(std::max<uint64_t>((per + 511) / 512 * 512, 512), kItemRowsMax);
    noalloc_setup_kernel<<<1, 1, 0, s>>>(st, build, prefix, ctl, n_rows, uint32_t(per), nfb);
    CK(cudaGetLastError());
    TrainerDev a{};
    a.bins = bins;  // column-blocked [nfb][dataset_rows][32]
    a.bins_row_stride = kBlockFeatures;
    a.bins_block_stride = uint64_t(dataset_rows) * kBlockFeatures;
    a.sm_count = uint32_t(sc.sm_count);
    a.n_rows = dataset_rows;
    a.seg_stride = dataset_rows;  // one segment (tree 0, parity 0) at offset 0
    a.features = features;
    a.nfb = nfb;
    a.n_trees = 1;
    a.rows = const_cast<uint32_t*>(rows);
    a.gh = const_cast<float2*>(gh);
    a.trees = st;
    a.hist = slot;
    a.n_slots = 1;
    a.build = build;
    a.build_prefix = prefix;
    a.ctl = ctl;
    a.item_rows = uint32_t(per);
    a.mode = kModeFixed;
    CK(launch_hist_build(a, HistConfig{}, sc.sm_count, s));
    const uint32_t cells = features * kSlots;
    noalloc_decode_kernel<<<std::max(1u, std::min(4096u, (cells + 255) / 256)), 256, 0, s>>>(
        slot, st, ctl, cells, out);
    CK(cudaGetLastError());
  });
}
