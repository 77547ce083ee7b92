// Quantile binning on the device: QuantizeDense / TransformDense
// (src/core/binned_dataset.cpp:95-238) for a matrix that then stays resident.
//
// Semantics (the same as the host restatement in quantize.cpp): NaN is missing (bin 0 plus
// a missing flag); Inf is an error; float64 input must fit float32. Per feature, with m
// non-missing values and desired = min(max_bins, m), the boundary candidates are the
// order statistics at ranks ceil(part * m / desired) - 1 for part = 1..desired-1, kept
// when below the maximum and above the previous kept boundary; a value's bin is the
// number of boundaries below it (lower_bound).
//
// No sort: the order statistics come from a three-round radix selection over the 32-bit
// order-preserving image of each float (11 + 11 + 10 bits). Round one histograms the top
// 11 bits of every value of a feature; each target rank then names its bucket, and the
// next round histograms the middle 11 bits of the values in those buckets only (at most
// 256 target buckets per feature), and so on. Three passes over the column, shared- and
// global-memory counters, and a per-feature selection block between passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "host_types.h"

using namespace mpsb;

namespace {

constexpr int kTargets = 256;        // at most max_bins order statistics per feature
constexpr uint32_t kNoSlot = 0xFFFFu;
constexpr uint32_t kErrInf = 1u;      // an Inf in the input
constexpr uint32_t kErrRange = 2u;    // a float64 value outside the float32 range

// Order-preserving image of a float: unsigned order of keys = numeric order of values
// (-0 sorts just below +0; both compare equal as floats, see the transform).
__device__ __forceinline__ uint32_t order_key(float x) {
  const uint32_t b = __float_as_uint(x);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_value(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__device__ __forceinline__ uint64_t quantile_rank(uint64_t part, uint64_t total, uint64_t divisor) {
  const uint64_t whole = part * (total / divisor);  // binned_dataset.cpp:83-95
  const uint64_t numerator = part * (total % divisor);
  return whole + numerator / divisor + (numerator % divisor != 0 ? 1 : 0) - 1;
}

// Input element (row, feature) at byte offset row * rs + feature * cs; returns false with
// an error bit for values the reference rejects.
__device__ __forceinline__ float load_value(const uint8_t* data, int scalar_type, uint64_t rs,
                                            uint64_t cs, uint64_t r, uint32_t f, uint32_t* err) {
  const uint8_t* p = data + r * rs + uint64_t(f) * cs;
  if (scalar_type == 1) {
    float x;
    memcpy(&x, p, sizeof x);
    if (isinf(x)) *err |= kErrInf;
    return x;
  }
  double x;
  memcpy(&x, p, sizeof x);
  if (isnan(x)) return __uint_as_float(0x7FC00000u);
  if (isinf(x)) {
    *err |= kErrInf;
    return 0.0f;
  }
  if (x > 3.4028234663852886e38 || x < -3.4028234663852886e38) *err |= kErrRange;
  return float(x);  // correctly rounded, as the host's static_cast
}

// Input matrix -> feature-major order keys and missing flags, through a 32 x 32 tile so
// both the row-major reads and the feature-major writes are coalesced.
__global__ void keys_kernel(const uint8_t* data, int scalar_type, uint64_t rs, uint64_t cs,
                            uint32_t n, uint32_t features, uint32_t* keys, uint8_t* missing,
                            unsigned long long* miss_count, uint32_t* error) {
  __shared__ float tile[32][33];
  __shared__ uint32_t miss[32];
  if (threadIdx.y == 0) miss[threadIdx.x] = 0;
  const uint32_t r0 = blockIdx.x * 32, f0 = blockIdx.y * 32;
  uint32_t err = 0;
  // Lanes walk the matrix's contiguous direction: features for row-major input, rows for
  // column-major input (the tile is indexed [row][feature] either way).
  const bool row_major = cs < rs;
  for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
    const uint32_t r = row_major ? r0 + i : r0 + threadIdx.x;
    const uint32_t f = row_major ? f0 + threadIdx.x : f0 + i;
    const float v = (r < n && f < features) ? load_value(data, scalar_type, rs, cs, r, f, &err) : 0.0f;
    if (row_major) tile[i][threadIdx.x] = v;
    else tile[threadIdx.x][i] = v;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
    const uint32_t f = f0 + i, r = r0 + threadIdx.x;
    if (f < features && r < n) {
      const float x = tile[threadIdx.x][i];
      const size_t o = size_t(f) * n + r;
      keys[o] = order_key(x);
      missing[o] = isnan(x) ? 1 : 0;
      if (isnan(x)) atomicAdd(&miss[i], 1u);
    }
  }
  if (err) atomicOr(error, err);
  __syncthreads();
  if (threadIdx.y == 0 && miss[threadIdx.x] && f0 + threadIdx.x < features)
    atomicAdd(&miss_count[f0 + threadIdx.x], (unsigned long long)miss[threadIdx.x]);
}

// Round one: per-feature histogram of the top 11 key bits of the non-missing values.
__global__ void hist_top_kernel(const uint32_t* keys, const uint8_t* missing, uint32_t n,
                                uint32_t* hist1) {
  __shared__ uint32_t sh[2048];
  const uint32_t f = blockIdx.y;
  for (uint32_t i = threadIdx.x; i < 2048; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const size_t base = size_t(f) * n;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    if (!missing[base + r]) atomicAdd(&sh[keys[base + r] >> 21], 1u);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < 2048; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist1[size_t(f) * 2048 + i], sh[i]);
}

// Per feature selection state between rounds.
struct Select {
  uint32_t m;                  // non-missing values
  uint32_t n_targets;          // desired (ranks of parts 1..desired-1, then the maximum)
  uint32_t rank[kTargets];     // residual rank inside the current bucket
  uint32_t prefix[kTargets];   // key bits chosen so far
  uint16_t slot[kTargets];     // bucket slot of the current round
  uint16_t n_slots;
};

// Block scan of 2048 counters held 8 per thread (256 threads): exclusive prefix in place.
__device__ void scan2048(uint32_t* c, uint32_t* total) {
  __shared__ uint32_t part[256];
  const int t = threadIdx.x;
  uint32_t v[8], s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[k] = c[t * 8 + k];
    s += v[k];
  }
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 256; off <<= 1) {
    const uint32_t y = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += y;
    __syncthreads();
  }
  uint32_t run = part[t] - s;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    c[t * 8 + k] = run;
    run += v[k];
  }
  if (t == 255) *total = part[255];
  __syncthreads();
}

// After round one: targets, their top-11-bit buckets and residual ranks, slots of the
// distinct buckets (ranks are non-decreasing, so equal buckets are adjacent).
__global__ void __launch_bounds__(256) select_top_kernel(const uint32_t* hist1, uint32_t max_bins,
                                                         Select* sel, uint16_t* slot1) {
  __shared__ uint32_t c[2048];
  __shared__ uint32_t total;
  __shared__ uint32_t bucket[kTargets];
  const uint32_t f = blockIdx.x;
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) c[i] = hist1[size_t(f) * 2048 + i];
  __syncthreads();
  scan2048(c, &total);
  Select& S = sel[f];
  const uint32_t m = total;
  const uint32_t desired = m < max_bins ? m : max_bins;
  if (threadIdx.x == 0) {
    S.m = m;
    S.n_targets = desired;
  }
  const uint32_t j = threadIdx.x;
  if (j < desired) {
    const uint32_t rank = j + 1 < desired ? uint32_t(quantile_rank(j + 1, m, desired)) : m - 1;
    uint32_t lo = 0, hi = 2048;  // last bucket whose prefix <= rank
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (c[mid] <= rank) lo = mid; else hi = mid;
    }
    bucket[j] = lo;
    S.rank[j] = rank - c[lo];
    S.prefix[j] = lo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint16_t s = 0;
    for (uint32_t k = 0; k < desired; ++k) {
      if (k > 0 && bucket[k] != bucket[k - 1]) ++s;
      S.slot[k] = s;
      slot1[size_t(f) * 2048 + bucket[k]] = s;
    }
    S.n_slots = desired ? uint16_t(s + 1) : 0;
  }
}

// Rounds two and three: histogram of the next digit of the values whose higher digits
// select a target slot. level 1: middle 11 bits under slot1; level 2: low 10 bits under
// (slot1, slot2).
template <int LEVEL>
__global__ void hist_next_kernel(const uint32_t* keys, const uint8_t* missing, uint32_t n,
                                 const uint16_t* slot1, const uint16_t* slot2, uint32_t* hist) {
  const uint32_t f = blockIdx.y;
  const size_t base = size_t(f) * n;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    if (missing[base + r]) continue;
    const uint32_t k = keys[base + r];
    const uint32_t s1 = slot1[size_t(f) * 2048 + (k >> 21)];
    if (s1 == kNoSlot) continue;
    if (LEVEL == 1) {
      atomicAdd(&hist[(size_t(f) * kTargets + s1) * 2048 + ((k >> 10) & 0x7FFu)], 1u);
    } else {
      const uint32_t s2 = slot2[(size_t(f) * kTargets + s1) * 2048 + ((k >> 10) & 0x7FFu)];
      if (s2 == kNoSlot) continue;
      atomicAdd(&hist[(size_t(f) * kTargets + s2) * 1024 + (k & 0x3FFu)], 1u);
    }
  }
}

// Selection of rounds two and three: each target walks its slot's digit histogram.
template <int LEVEL>
__global__ void __launch_bounds__(256) select_next_kernel(const uint32_t* hist, Select* sel,
                                                          uint16_t* slot2) {
  constexpr uint32_t D = LEVEL == 1 ? 2048 : 1024;
  constexpr int SHIFT = LEVEL == 1 ? 11 : 10;
  __shared__ uint32_t digit[kTargets];
  const uint32_t f = blockIdx.x;
  Select& S = sel[f];
  const uint32_t j = threadIdx.x;
  const uint32_t nt = S.n_targets;
  if (j < nt) {
    const uint32_t* h = hist + (size_t(f) * kTargets + S.slot[j]) * D;
    uint32_t rank = S.rank[j], d = 0;
    for (; d + 1 < D; ++d) {
      const uint32_t c = h[d];
      if (rank < c) break;
      rank -= c;
    }
    digit[j] = d;
    S.rank[j] = rank;
    S.prefix[j] = (S.prefix[j] << SHIFT) | d;
  }
  __syncthreads();
  if (LEVEL == 1 && threadIdx.x == 0) {  // slots of the distinct (top, middle) prefixes
    uint16_t s = 0;
    for (uint32_t k = 0; k < nt; ++k) {
      if (k > 0 && S.prefix[k] != S.prefix[k - 1]) ++s;
      slot2[(size_t(f) * kTargets + S.slot[k]) * 2048 + digit[k]] = s;
      S.slot[k] = s;
    }
  }
}

// Boundaries from the selected order statistics (BuildBoundaries, binned_dataset.cpp:97-118).
__global__ void finish_kernel(const Select* sel, uint32_t features, float* bounds, uint32_t* counts) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= features) return;
  const Select& S = sel[f];
  uint32_t count = 0;
  if (S.n_targets > 0) {
    const float maximum = key_value(S.prefix[S.n_targets - 1]);
    for (uint32_t k = 0; k + 1 < S.n_targets; ++k) {
      const float c = key_value(S.prefix[k]);
      if (c < maximum && (count == 0 || c > bounds[size_t(f) * kTargets + count - 1]))
        bounds[size_t(f) * kTargets + count++] = c;
    }
  }
  counts[f] = count;
}

// bin = lower_bound(boundaries, value) in float order (so -0 and +0 bin alike); missing
// rows get bin 0 (their flag marks them).
__global__ void transform_kernel(const uint32_t* keys, const uint8_t* missing, uint32_t n,
                                 const float* bounds, const uint32_t* counts, uint8_t* bins) {
  __shared__ float b[kTargets];
  const uint32_t f = blockIdx.y;
  const uint32_t nb = counts[f];
  for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) b[i] = bounds[size_t(f) * kTargets + i];
  __syncthreads();
  const size_t base = size_t(f) * n;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    uint32_t bin = 0;
    if (!missing[base + r]) {
      const float x = key_value(keys[base + r]);
      uint32_t lo = 0, hi = nb;  // first boundary not less than x
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (b[mid] < x) lo = mid + 1; else hi = mid;
      }
      bin = lo;
    }
    bins[base + r] = uint8_t(bin);
  }
}

struct Scratch {
  std::vector<std::unique_ptr<DevBuf>> bufs;
  template <class T>
  T* alloc(size_t count) {
    bufs.emplace_back(new DevBuf);
    bufs.back()->alloc(count * sizeof(T));
    return bufs.back()->as<T>();
  }
};

void check_view(const void* data, int scalar_type, uint64_t rows, uint32_t features, uint64_t rs,
                uint64_t cs, uint64_t* extent) {
  if (data == nullptr) throw DataError("Input matrix data must not be null");
  if (rows == 0 || features == 0) throw DataError("Input matrix must contain at least one row and one feature");
  if (scalar_type != 1 && scalar_type != 2) throw DataError("Input scalar type is not supported");
  if (rows >= 0xFFFFFFFFull) throw UnsupportedError("the CUDA backend indexes rows with uint32");
  const uint64_t item = scalar_type == 2 ? 8 : 4;
  if (rs < item || cs < item) throw DataError("Input matrix stride is smaller than the element size");
  uint64_t a, b, c;
  if (__builtin_mul_overflow(rows - 1, rs, &a) || __builtin_mul_overflow(uint64_t(features - 1), cs, &b) ||
      __builtin_add_overflow(a, b, &c) || __builtin_add_overflow(c, item, &c))
    throw DataError("input matrix maximum offset: multiplication overflow");
  *extent = c;
}

// Upload the matrix and turn it into keys + missing flags.
void make_keys(mpsb_cuda_backend* b, Scratch& ss, const void* data, int scalar_type, uint64_t rows,
               uint32_t features, uint64_t rs, uint64_t cs, uint32_t** keys, uint8_t** missing,
               std::vector<uint64_t>* missing_count) {
  uint64_t extent = 0;
  check_view(data, scalar_type, rows, features, rs, cs, &extent);
  cudaStream_t s = b->stream;
  uint8_t* raw = ss.alloc<uint8_t>(extent);
  CK(cudaMemcpyAsync(raw, data, extent, cudaMemcpyHostToDevice, s));
  const size_t cells = size_t(rows) * features;
  *keys = ss.alloc<uint32_t>(cells);
  *missing = ss.alloc<uint8_t>(cells);
  unsigned long long* miss = ss.alloc<unsigned long long>(features);
  CK(cudaMemsetAsync(miss, 0, features * sizeof(unsigned long long), s));
  CK(cudaMemsetAsync(b->error.p, 0, sizeof(uint32_t), s));
  const dim3 grid(uint32_t((rows + 31) / 32), (features + 31) / 32);
  keys_kernel<<<grid, dim3(32, 8), 0, s>>>(raw, scalar_type, rs, cs, uint32_t(rows), features, *keys,
                                             *missing, miss, b->error.as<uint32_t>());
  CK(cudaGetLastError());
  missing_count->assign(features, 0);
  CK(cudaMemcpyAsync(missing_count->data(), miss, features * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  const uint32_t e = b->take_error();  // synchronizes the stream
  if (e & kErrInf) throw DataError("Input matrix contains Inf");
  if (e & kErrRange) throw DataError("float64 input value exceeds the finite float32 range");
}

// Build the resident dataset from feature-major bins (u8 or u16: `width` bytes) and
// missing flags on the device.
mpsb_cuda_dataset* finish_dataset(mpsb_cuda_backend* b, const void* bins_fm, uint32_t width,
                                  const uint8_t* missing, uint32_t rows, uint32_t features,
                                  std::vector<uint32_t> bin_count, std::vector<uint64_t> missing_count) {
  cudaStream_t s = b->stream;
  std::unique_ptr<mpsb_cuda_dataset> d(new mpsb_cuda_dataset);
  d->backend = b;
  d->n_rows = rows;
  d->features = features;
  d->nfb = (features + kBlockFeatures - 1) / kBlockFeatures;
  d->h_bin_count = std::move(bin_count);
  d->h_has_missing.assign(features, 0);
  for (uint32_t f = 0; f < features; ++f) d->h_has_missing[f] = missing_count[f] ? 1 : 0;
  // 256 bins and missing values in one feature: the wide layout's missing slot.
  d->slots = dataset_slots(d->h_bin_count.data(), d->h_has_missing.data(), features);
  d->missing_count = std::move(missing_count);
  d->bin_count.alloc(features * sizeof(uint32_t));
  d->has_missing.alloc(features);
  CK(cudaMemcpyAsync(d->bin_count.p, d->h_bin_count.data(), features * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d->has_missing.p, d->h_has_missing.data(), features, cudaMemcpyHostToDevice, s));
  if (d->slots != uint32_t(kSlots)) {
    d->bins16.alloc(size_t(d->nfb) * rows * kBlockFeatures * sizeof(uint16_t));
    d->bins16_fm.alloc(size_t(features) * rows * sizeof(uint16_t));
    for (uint32_t fb = 0; fb < d->nfb; ++fb) {
      const size_t first = size_t(fb) * kBlockFeatures * rows;
      CK(launch_pack_bins16_block(static_cast<const uint8_t*>(bins_fm) + first * width, width,
                                  missing ? missing + first : nullptr,
                                  d->bin_count.as<uint32_t>(), rows,
                                  features, fb, d->slots, d->bins16.as<uint16_t>(),
                                  d->bins16_fm.as<uint16_t>(), b->error.as<uint32_t>(), s));
    }
  } else {
    d->bins.alloc(size_t(d->nfb) * rows * kBlockFeatures);
    d->bins_blocked.alloc(size_t(d->nfb) * rows * kBlockFeatures);
    d->bins_fm.alloc(size_t(features) * rows);
    CK(launch_pack_bins(bins_fm, width, missing, d->bin_count.as<uint32_t>(), rows, features, d->nfb,
                        d->bins.as<uint8_t>(), d->bins_blocked.as<uint8_t>(), d->bins_fm.as<uint8_t>(),
                        b->error.as<uint32_t>(), s));
  }
  if (b->take_error()) throw DataError("Binned value exceeds the feature histogram range");
  attach_bins_tmap(d.get());
  return d.release();
}

// ---- More than 256 bins per feature -------------------------------------------------
// The selection above keeps one target slot per boundary (at most 256). Wide schemas
// sort each feature's order keys instead (a stable LSD radix sort, eight passes of 4-bit
// digits, every feature in the same launches) and read the order statistics at their
// ranks; missing rows carry the key 0xFFFFFFFF, above every finite value's, so they sort
// last and the first m keys of a feature are its non-missing values in order.
constexpr int kSortThreads = 256;
constexpr uint32_t kSortTile = 4096;  // keys per (feature, tile) block
constexpr uint32_t kMissingKey = 0xFFFFFFFFu;

__global__ void sort_keys_init_kernel(const uint32_t* keys, const uint8_t* missing, size_t cells,
                                      uint32_t* out) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < cells; i += size_t(gridDim.x) * blockDim.x)
    out[i] = missing[i] ? kMissingKey : keys[i];
}

// Digit counts of one (tile, feature): cnt[(f * 16 + digit) * tiles + tile].
__global__ void __launch_bounds__(kSortThreads) sort_count_kernel(const uint32_t* keys, uint32_t n,
                                                                  uint32_t tiles, int shift, uint32_t* cnt) {
  __shared__ uint32_t c[16];
  const uint32_t f = blockIdx.y, t = blockIdx.x;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 16) c[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t* k = keys + size_t(f) * n;
  const uint32_t lo = t * kSortTile, hi = min(n, lo + kSortTile);
  uint32_t mine = 0;  // lane v < 16 counts digit v for its warp
  for (uint32_t base = lo + (threadIdx.x & ~31u); base < hi; base += kSortThreads) {
    const uint32_t i = base + uint32_t(lane);
    const bool valid = i < hi;
    const uint32_t d = valid ? (k[i] >> shift) & 15u : 16u;
#pragma unroll
    for (uint32_t v = 0; v < 16; ++v) {
      const uint32_t m = __ballot_sync(0xffffffffu, d == v);
      if (uint32_t(lane) == v) mine += uint32_t(__popc(m));
    }
  }
  if (lane < 16 && mine) atomicAdd(&c[lane], mine);
  __syncthreads();
  if (threadIdx.x < 16) cnt[(size_t(f) * 16 + threadIdx.x) * tiles + t] = c[threadIdx.x];
}

// Exclusive prefix of one feature's counts in (digit, tile) order, in place.
__global__ void __launch_bounds__(1024) sort_scan_kernel(uint32_t* cnt, uint32_t tiles) {
  __shared__ uint32_t warp_sum[32];
  __shared__ uint32_t carry;
  const uint32_t f = blockIdx.x;
  uint32_t* c = cnt + size_t(f) * 16 * tiles;
  const uint32_t total = 16 * tiles;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < total; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < total ? c[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      const uint32_t w = lane < int(blockDim.x >> 5) ? warp_sum[lane] : 0u;
      uint32_t z = w;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, z, off);
        if (lane >= off) z += y;
      }
      warp_sum[lane] = z - w;  // exclusive
    }
    __syncthreads();
    const uint32_t before = carry;
    if (i < total) c[i] = before + warp_sum[warp] + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + warp_sum[warp] + x;
    __syncthreads();
  }
}

// Stable scatter of one (tile, feature) by the digit at `shift`: the tile's keys in
// rounds of kSortThreads; a key's place is its digit's offset for the tile, plus the
// earlier keys of the tile with that digit (previous rounds, earlier warps of the round,
// lower lanes of its warp).
__global__ void __launch_bounds__(kSortThreads) sort_scatter_kernel(const uint32_t* in, uint32_t* out,
                                                                    uint32_t n, uint32_t tiles, int shift,
                                                                    const uint32_t* off) {
  constexpr int W = kSortThreads / 32;
  __shared__ uint32_t run[16];
  __shared__ uint32_t wcount[W][16];
  const uint32_t f = blockIdx.y, t = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < 16) run[threadIdx.x] = off[(size_t(f) * 16 + threadIdx.x) * tiles + t];
  const uint32_t* k = in + size_t(f) * n;
  uint32_t* o = out + size_t(f) * n;
  const uint32_t lo = t * kSortTile, hi = min(n, lo + kSortTile);
  const uint32_t lt = (1u << lane) - 1u;
  __syncthreads();
  for (uint32_t base = lo; base < hi; base += kSortThreads) {
    const uint32_t i = base + threadIdx.x;
    const bool valid = i < hi;
    const uint32_t key = valid ? k[i] : 0u;
    const uint32_t d = valid ? (key >> shift) & 15u : 16u;
    uint32_t rank = 0;
#pragma unroll
    for (uint32_t v = 0; v < 16; ++v) {
      const uint32_t m = __ballot_sync(0xffffffffu, d == v);
      if (d == v) rank = uint32_t(__popc(m & lt));
      if (uint32_t(lane) == v) wcount[warp][v] = uint32_t(__popc(m));
    }
    __syncthreads();
    if (valid) {
      uint32_t before = run[d] + rank;
      for (int w = 0; w < warp; ++w) before += wcount[w][d];
      if (before < n) o[before] = key;  // always: the counts come from the same keys
    }
    __syncthreads();
    if (threadIdx.x < 16) {
      uint32_t sum = 0;
      for (int w = 0; w < W; ++w) sum += wcount[w][threadIdx.x];
      run[threadIdx.x] += sum;
    }
    __syncthreads();
  }
}

// Boundaries of one feature from its sorted keys (BuildBoundaries, binned_dataset.cpp:
// 97-118): candidate p (1 <= p < desired) is the value at rank QuantileRank(p, m, desired)
// and is kept when below the maximum and above the previous candidate. The candidates are
// non-decreasing, so "above the last kept boundary" is "above the previous candidate" for
// every candidate below the maximum. A block per feature; kept candidates are compacted
// in order by a block prefix sum.
__global__ void __launch_bounds__(1024) wide_bounds_kernel(const uint32_t* sorted, uint32_t n,
                                                           const uint64_t* miss_count, uint32_t max_bins,
                                                           float* bounds, uint32_t* counts) {
  __shared__ uint32_t warp_sum[32];
  __shared__ uint32_t carry;
  const uint32_t f = blockIdx.x;
  const uint32_t* k = sorted + size_t(f) * n;
  const uint32_t m = n - uint32_t(miss_count[f]);
  const uint32_t desired = m < max_bins ? m : max_bins;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const float maximum = m ? key_value(k[m - 1]) : 0.0f;
  const uint32_t parts = desired > 1 ? desired - 1 : 0;  // candidates p = 1 .. desired - 1
  float* out = bounds + size_t(f) * (max_bins - 1);
  for (uint32_t base = 0; base < parts; base += blockDim.x) {
    const uint32_t p = base + threadIdx.x + 1;
    bool keep = false;
    float c = 0.0f;
    if (p <= parts) {
      c = key_value(k[quantile_rank(p, m, desired)]);
      keep = c < maximum && (p == 1 || c > key_value(k[quantile_rank(p - 1, m, desired)]));
    }
    const uint32_t ballot = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_sum[warp] = uint32_t(__popc(ballot));
    __syncthreads();
    if (warp == 0) {
      const uint32_t w = lane < int(blockDim.x >> 5) ? warp_sum[lane] : 0u;
      uint32_t z = w;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, z, off);
        if (lane >= off) z += y;
      }
      warp_sum[lane] = z - w;
    }
    __syncthreads();
    const uint32_t before = carry;
    if (keep) out[before + warp_sum[warp] + uint32_t(__popc(ballot & ((1u << lane) - 1u)))] = c;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + warp_sum[warp] + uint32_t(__popc(ballot));
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[f] = carry;
}

// Wide transform: bin = lower_bound over the feature's boundaries (global memory, up to
// 65535 per feature at bounds + f * stride); missing rows get bin 0 (their flag marks them).
__global__ void transform_wide_kernel(const uint32_t* keys, const uint8_t* missing, uint32_t n,
                                      const float* bounds, size_t stride, const uint32_t* counts,
                                      uint16_t* bins) {
  const uint32_t f = blockIdx.y;
  const uint32_t nb = counts[f];
  const float* b = bounds + size_t(f) * stride;
  const size_t base = size_t(f) * n;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    uint32_t bin = 0;
    if (!missing[base + r]) {
      const float x = key_value(keys[base + r]);
      uint32_t lo = 0, hi = nb;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(b + mid) < x) lo = mid + 1; else hi = mid;
      }
      bin = lo;
    }
    bins[base + r] = uint16_t(bin);
  }
}

// Sorts every feature's keys (missing rows last) into `sorted`; `tmp` is a buffer of the
// same size. Eight passes: the result ends where it started.
void sort_feature_keys(cudaStream_t s, Scratch& ss, const uint32_t* keys, const uint8_t* missing,
                       uint32_t n, uint32_t features, uint32_t* sorted, uint32_t* tmp) {
  const size_t cells = size_t(n) * features;
  const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
  uint32_t* cnt = ss.alloc<uint32_t>(size_t(features) * 16 * tiles);
  sort_keys_init_kernel<<<unsigned(std::min<size_t>((cells + 255) / 256, 152 * 32)), 256, 0, s>>>(
      keys, missing, cells, sorted);
  CK(cudaGetLastError());
  uint32_t* a = sorted;
  uint32_t* b = tmp;
  for (int shift = 0; shift < 32; shift += 4) {
    sort_count_kernel<<<dim3(tiles, features), kSortThreads, 0, s>>>(a, n, tiles, shift, cnt);
    CK(cudaGetLastError());
    sort_scan_kernel<<<features, 1024, 0, s>>>(cnt, tiles);
    CK(cudaGetLastError());
    sort_scatter_kernel<<<dim3(tiles, features), kSortThreads, 0, s>>>(a, b, n, tiles, shift, cnt);
    CK(cudaGetLastError());
    std::swap(a, b);
  }
}

// QuantizeDense for max_bins > 256 on the device: u16 feature-major bins in `bins_fm`,
// boundaries [features][max_bins - 1] in `bounds` with their counts.
void quantize_wide(cudaStream_t s, Scratch& ss, const uint32_t* keys, const uint8_t* missing,
                   const std::vector<uint64_t>& missing_count, uint32_t n, uint32_t features,
                   uint32_t max_bins, float* bounds, uint32_t* counts, uint16_t* bins_fm) {
  const size_t cells = size_t(n) * features;
  uint32_t* sorted = ss.alloc<uint32_t>(cells);
  uint32_t* tmp = ss.alloc<uint32_t>(cells);
  sort_feature_keys(s, ss, keys, missing, n, features, sorted, tmp);
  uint64_t* d_miss = ss.alloc<uint64_t>(features);
  CK(cudaMemcpyAsync(d_miss, missing_count.data(), features * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  wide_bounds_kernel<<<features, 1024, 0, s>>>(sorted, n, d_miss, max_bins, bounds, counts);
  CK(cudaGetLastError());
}

// The device's feature-major copy as the reference lays bins out: missing rows (at the
// dataset's missing slot) become bin 0 plus a flag.
template <typename T>
void export_bins(const mpsb_cuda_dataset* d, T* bins, uint8_t* missing) {
  dataset_ready(d);
  d->backend->activate();
  cudaStream_t s = d->backend->stream;
  const size_t cells = size_t(d->n_rows) * d->features;
  const bool wide = d->slots != uint32_t(kSlots);
  std::vector<uint16_t> b16(wide ? cells : 0);
  std::vector<uint8_t> b8(wide ? 0 : cells);
  if (wide)
    CK(cudaMemcpyAsync(b16.data(), d->bins16_fm.p, cells * sizeof(uint16_t), cudaMemcpyDeviceToHost, s));
  else
    CK(cudaMemcpyAsync(b8.data(), d->bins_fm.p, cells, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const uint32_t missing_slot = d->slots - 1;
  for (uint32_t f = 0; f < d->features; ++f) {
    for (uint32_t r = 0; r < d->n_rows; ++r) {
      const size_t i = size_t(f) * d->n_rows + r;
      const uint32_t v = wide ? uint32_t(b16[i]) : uint32_t(b8[i]);
      const bool miss = d->h_has_missing[f] && v == missing_slot;
      if (missing) missing[i] = miss ? 1 : 0;
      bins[i] = T(miss ? 0u : v);
    }
  }
}

}  // namespace

extern "C" {

int mpsb_cuda_dataset_quantize(mpsb_cuda_backend* b, const void* data, int scalar_type,
                               uint64_t rows, uint32_t features, uint64_t row_stride,
                               uint64_t col_stride, uint32_t max_bins, mpsb_cuda_dataset** out) {
  return guard([&] {
    if (!b || !out) throw TrainingError("null argument");
    if (max_bins < 2 || max_bins > 65536) throw DataError("max_bins must be in [2, 65536]");
    if (features > 65535) throw UnsupportedError("device binning takes at most 65535 features");
    b->activate();
    cudaStream_t s = b->stream;
    Scratch ss;
    uint32_t* keys = nullptr;
    uint8_t* missing = nullptr;
    std::vector<uint64_t> missing_count;
    make_keys(b, ss, data, scalar_type, rows, features, row_stride, col_stride, &keys, &missing,
              &missing_count);
    const uint32_t n = uint32_t(rows);
    // Schema on the host: per feature the boundary count and `stride` boundary slots.
    std::vector<uint32_t> h_counts(features);
    std::vector<float> h_bounds;
    size_t stride = 0;
    std::unique_ptr<mpsb_cuda_dataset> d;
    if (max_bins > uint32_t(kTargets)) {
      stride = max_bins - 1;
      float* bounds = ss.alloc<float>(size_t(features) * stride);
      uint32_t* counts = ss.alloc<uint32_t>(features);
      uint16_t* bins16 = ss.alloc<uint16_t>(size_t(features) * n);
      quantize_wide(s, ss, keys, missing, missing_count, n, features, max_bins, bounds, counts, bins16);
      const dim3 grid(std::max(1u, std::min((n + 255) / 256, uint32_t(b->sm_count) * 4 / std::max(1u, features) + 1)),
                      features);
      transform_wide_kernel<<<grid, 256, 0, s>>>(keys, missing, n, bounds, stride, counts, bins16);
      CK(cudaGetLastError());
      h_bounds.resize(size_t(features) * stride);
      CK(cudaMemcpyAsync(h_counts.data(), counts, features * 4, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(h_bounds.data(), bounds, h_bounds.size() * 4, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      std::vector<uint32_t> bin_count(features);
      for (uint32_t f = 0; f < features; ++f) bin_count[f] = h_counts[f] + 1;
      d.reset(finish_dataset(b, bins16, 2, missing, n, features, bin_count, missing_count));
    } else {
      uint32_t* hist1 = ss.alloc<uint32_t>(size_t(features) * 2048);
      uint32_t* hist2 = ss.alloc<uint32_t>(size_t(features) * kTargets * 2048);
      uint32_t* hist3 = ss.alloc<uint32_t>(size_t(features) * kTargets * 1024);
      uint16_t* slot1 = ss.alloc<uint16_t>(size_t(features) * 2048);
      uint16_t* slot2 = ss.alloc<uint16_t>(size_t(features) * kTargets * 2048);
      Select* sel = ss.alloc<Select>(features);
      float* bounds = ss.alloc<float>(size_t(features) * kTargets);
      uint32_t* counts = ss.alloc<uint32_t>(features);
      uint8_t* bins_fm = ss.alloc<uint8_t>(size_t(features) * n);
      CK(cudaMemsetAsync(hist1, 0, size_t(features) * 2048 * 4, s));
      CK(cudaMemsetAsync(hist2, 0, size_t(features) * kTargets * 2048 * 4, s));
      CK(cudaMemsetAsync(hist3, 0, size_t(features) * kTargets * 1024 * 4, s));
      CK(cudaMemsetAsync(slot1, 0xFF, size_t(features) * 2048 * 2, s));
      CK(cudaMemsetAsync(slot2, 0xFF, size_t(features) * kTargets * 2048 * 2, s));
      const dim3 grid(std::max(1u, std::min((n + 255) / 256, uint32_t(b->sm_count) * 4 / std::max(1u, features) + 1)),
                      features);
      hist_top_kernel<<<grid, 256, 0, s>>>(keys, missing, n, hist1);
      CK(cudaGetLastError());
      select_top_kernel<<<features, 256, 0, s>>>(hist1, max_bins, sel, slot1);
      CK(cudaGetLastError());
      hist_next_kernel<1><<<grid, 256, 0, s>>>(keys, missing, n, slot1, slot2, hist2);
      CK(cudaGetLastError());
      select_next_kernel<1><<<features, 256, 0, s>>>(hist2, sel, slot2);
      CK(cudaGetLastError());
      hist_next_kernel<2><<<grid, 256, 0, s>>>(keys, missing, n, slot1, slot2, hist3);
      CK(cudaGetLastError());
      select_next_kernel<2><<<features, 256, 0, s>>>(hist3, sel, slot2);
      CK(cudaGetLastError());
      finish_kernel<<<(features + 127) / 128, 128, 0, s>>>(sel, features, bounds, counts);
      CK(cudaGetLastError());
      transform_kernel<<<grid, 256, 0, s>>>(keys, missing, n, bounds, counts, bins_fm);
      CK(cudaGetLastError());
      // Schema back to the host.
      stride = kTargets;
      h_bounds.resize(size_t(features) * kTargets);
      std::vector<Select> h_sel(features);
      CK(cudaMemcpyAsync(h_counts.data(), counts, features * 4, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(h_bounds.data(), bounds, h_bounds.size() * 4, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(h_sel.data(), sel, features * sizeof(Select), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      std::vector<uint32_t> bin_count(features);
      for (uint32_t f = 0; f < features; ++f) {
        bin_count[f] = h_counts[f] + 1;
        if (missing_count[f] + h_sel[f].m != rows) throw BackendError("device binning lost rows");
      }
      d.reset(finish_dataset(b, bins_fm, 1, missing, n, features, bin_count, missing_count));
    }
    d->max_bins = max_bins;
    d->boundary_offset.resize(features);
    uint64_t off = 0;
    for (uint32_t f = 0; f < features; ++f) {
      d->boundary_offset[f] = off;
      d->boundaries.insert(d->boundaries.end(), h_bounds.begin() + size_t(f) * stride,
                           h_bounds.begin() + size_t(f) * stride + h_counts[f]);
      off += h_counts[f];
    }
    d->boundary_count = h_counts;
    d->has_schema = true;
    *out = d.release();
  });
}

int mpsb_cuda_dataset_transform(mpsb_cuda_backend* b, const mpsb_cuda_dataset* schema,
                                const void* data, int scalar_type, uint64_t rows,
                                uint32_t features, uint64_t row_stride, uint64_t col_stride,
                                mpsb_cuda_dataset** out) {
  return guard([&] {
    if (!b || !schema || !out) throw TrainingError("null argument");
    dataset_ready(schema);
    if (!schema->has_schema) throw TrainingError("the schema dataset holds no bin boundaries");
    if (features != schema->features)
      throw DataError("Prediction input feature count does not match the binned schema");
    b->activate();
    cudaStream_t s = b->stream;
    Scratch ss;
    uint32_t* keys = nullptr;
    uint8_t* missing = nullptr;
    std::vector<uint64_t> missing_count;
    make_keys(b, ss, data, scalar_type, rows, features, row_stride, col_stride, &keys, &missing,
              &missing_count);
    const uint32_t n = uint32_t(rows);
    const bool wide = schema->max_bins > uint32_t(kTargets);
    const size_t stride = wide ? schema->max_bins - 1 : size_t(kTargets);
    std::vector<float> h_bounds(size_t(features) * stride, 0.0f);
    for (uint32_t f = 0; f < features; ++f)
      std::copy(schema->boundaries.begin() + schema->boundary_offset[f],
                schema->boundaries.begin() + schema->boundary_offset[f] + schema->boundary_count[f],
                h_bounds.begin() + size_t(f) * stride);
    float* bounds = ss.alloc<float>(h_bounds.size());
    uint32_t* counts = ss.alloc<uint32_t>(features);
    CK(cudaMemcpyAsync(bounds, h_bounds.data(), h_bounds.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(counts, schema->boundary_count.data(), features * 4, cudaMemcpyHostToDevice, s));
    const dim3 grid(std::max(1u, std::min((n + 255) / 256, uint32_t(b->sm_count) * 4 / std::max(1u, features) + 1)),
                    features);
    std::unique_ptr<mpsb_cuda_dataset> d;
    if (wide) {
      uint16_t* bins16 = ss.alloc<uint16_t>(size_t(features) * n);
      transform_wide_kernel<<<grid, 256, 0, s>>>(keys, missing, n, bounds, stride, counts, bins16);
      CK(cudaGetLastError());
      d.reset(finish_dataset(b, bins16, 2, missing, n, features, schema->h_bin_count, missing_count));
    } else {
      uint8_t* bins_fm = ss.alloc<uint8_t>(size_t(features) * n);
      transform_kernel<<<grid, 256, 0, s>>>(keys, missing, n, bounds, counts, bins_fm);
      CK(cudaGetLastError());
      d.reset(finish_dataset(b, bins_fm, 1, missing, n, features, schema->h_bin_count, missing_count));
    }
    d->max_bins = schema->max_bins;
    d->boundaries = schema->boundaries;
    d->boundary_offset = schema->boundary_offset;
    d->boundary_count = schema->boundary_count;
    d->has_schema = true;
    *out = d.release();
  });
}

uint64_t mpsb_cuda_dataset_boundary_total(const mpsb_cuda_dataset* d) {
  return d ? d->boundaries.size() : 0;
}

int mpsb_cuda_dataset_schema(const mpsb_cuda_dataset* d, float* boundaries,
                             uint64_t* boundary_offset, uint32_t* boundary_count,
                             uint32_t* bin_count, uint64_t* missing_count) {
  return guard([&] {
    if (!d) throw TrainingError("null argument");
    if (!d->has_schema) throw TrainingError("the dataset holds no bin boundaries");
    if (boundaries) std::copy(d->boundaries.begin(), d->boundaries.end(), boundaries);
    if (boundary_offset) std::copy(d->boundary_offset.begin(), d->boundary_offset.end(), boundary_offset);
    if (boundary_count) std::copy(d->boundary_count.begin(), d->boundary_count.end(), boundary_count);
    if (bin_count) std::copy(d->h_bin_count.begin(), d->h_bin_count.end(), bin_count);
    if (missing_count) std::copy(d->missing_count.begin(), d->missing_count.end(), missing_count);
  });
}

int mpsb_cuda_dataset_export(const mpsb_cuda_dataset* d, uint8_t* bins, uint8_t* missing) {
  return guard([&] {
    if (!d || !bins) throw TrainingError("null argument");
    for (uint32_t f = 0; f < d->features; ++f)
      if (d->h_bin_count[f] > 256)
        throw UnsupportedError("the dataset has more than 256 bins per feature: export it as u16");
    export_bins(d, bins, missing);
  });
}

int mpsb_cuda_dataset_export16(const mpsb_cuda_dataset* d, uint16_t* bins, uint8_t* missing) {
  return guard([&] {
    if (!d || !bins) throw TrainingError("null argument");
    export_bins(d, bins, missing);
  });
}

}  // extern "C"
