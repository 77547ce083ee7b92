// Histogram build for sm_103a: the hot kernel of the training path.
//
// Replaces the two-stage Metal histogram (src/mps/kernels/histogram.metal:34-182 driven
// by src/mps/mps_histogram.mm:82-256). Design:
//  * Bins are column-blocked u8, [feature_block][row][32]: one row of a block is one
//    32-byte sector, gathered with two 16-byte cp.async copies.
//  * Persistent CTAs (one per SM) pull work items (build node, row chunk <= 65536 rows,
//    feature block) from a device counter; every frontier node of every tree of a level
//    is in the same launch.
//  * A 3-stage cp.async pipeline stages the row ids' bin sectors and FP32 g/h pairs;
//    row ids are prefetched one tile ahead in registers.
//  * The CTA-private histogram lives in shared memory laid out [bin][feature]: in one
//    atomic instruction the 16 lanes of a half-warp update 16 different features of 16
//    different rows (feature index rotated by the row), so their words fall in 16
//    different bank pairs for any bin values: conflict-free shared atomics.
//  * Fixed mode: q_g = rne(g * 2^kg) accumulated as int64; q_h + 2^47 accumulated as one
//    int64 word, so count (bits 47..63) and the h-sum (bits 0..46, < 2^46 for <= 2^16
//    rows) need one atomic: two 64-bit shared atomics per cell. Exact and
//    order-independent. Float mode: u32 count + two FP32 atomics per cell.
//  * The CTA flushes its non-empty cells into the node's global slot with 64-bit
//    red.global adds (exact integer adds in fixed mode; FP64 adds in float mode).
#include "device.cuh"
#include "kernels.h"

namespace mpsb {
namespace {

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Rotate a 16-byte vector right by s bytes (s in [0, 16)): byte j of the result is byte
// (j + s) mod 16 of the input.
__device__ __forceinline__ uint4 rotate_bytes(uint4 v, uint32_t s) {
  const uint32_t ws = s >> 2, bs = (s & 3u) * 8u;
  uint32_t x0 = v.x, x1 = v.y, x2 = v.z, x3 = v.w;
  if (ws & 1u) { const uint32_t t = x0; x0 = x1; x1 = x2; x2 = x3; x3 = t; }
  if (ws & 2u) { uint32_t t = x0; x0 = x2; x2 = t; t = x1; x1 = x3; x3 = t; }
  uint4 r;
  r.x = __funnelshift_r(x0, x1, bs);
  r.y = __funnelshift_r(x1, x2, bs);
  r.z = __funnelshift_r(x2, x3, bs);
  r.w = __funnelshift_r(x3, x0, bs);
  return r;
}

template <int MODE>
struct HistSmem;

template <>
struct HistSmem<kModeFixed> {
  static constexpr size_t kBytes = 2ull * kSlots * kBlockFeatures * sizeof(long long);
};
template <>
struct HistSmem<kModeFloat> {
  static constexpr size_t kBytes = 3ull * kSlots * kBlockFeatures * sizeof(uint32_t);
};

template <int MODE, int THREADS, int NSTAGE>
__global__ void __launch_bounds__(THREADS, 1) hist_build_kernel(TrainerDev a) {
  constexpr int TILE = THREADS;
  constexpr int WARPS = THREADS / 32;
  constexpr int ROWS_PER_STEP = WARPS * 16;
  constexpr int CELLS = kSlots * kBlockFeatures;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* hist_smem = smem;
  uint4* stage_bins = reinterpret_cast<uint4*>(smem + HistSmem<MODE>::kBytes);  // [NSTAGE][TILE][2]
  float2* stage_gh = reinterpret_cast<float2*>(stage_bins + NSTAGE * TILE * 2);  // [NSTAGE][TILE]

  __shared__ uint32_t s_item, s_entry;

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t half = lane >> 4;
  const uint32_t r16 = lane & 15;
  const uint32_t n = a.n_rows;
  const uint32_t nfb = a.nfb;

  for (;;) {
    const uint32_t limit = a.item_end ? a.item_end : a.ctl->hist_items;
    if (tid == 0) {
      const uint32_t item = a.item_begin + atomicAdd(&a.ctl->hist_counter, 1u);
      s_item = item;
      if (item < limit) {
        const uint32_t chunk = item / nfb;
        uint32_t lo = 0, hi = a.ctl->n_build;  // last entry with prefix <= chunk
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (a.build_prefix[mid] <= chunk) lo = mid; else hi = mid;
        }
        s_entry = lo;
      }
    }
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= limit) break;
    const uint32_t fb = item % nfb;
    const uint32_t chunk = item / nfb;
    const BuildEntry e = a.build[s_entry];
    const uint32_t row_begin = (chunk - a.build_prefix[s_entry]) * a.item_rows;
    const uint32_t row_count = row_begin < e.seg_cnt ? min(a.item_rows, e.seg_cnt - row_begin) : 0u;
    const uint32_t* rows = a.rows + (size_t(e.tree) * 2 + e.parity) * n + e.seg_off + row_begin;
    const float2* gh = a.gh + size_t(e.tree) * n;
    const uint8_t* bins = a.bins + size_t(fb) * n * kBlockFeatures;
    const int kg = a.trees[e.tree].kg;
    const int kh = a.trees[e.tree].kh;

    // Zero the CTA histogram.
    {
      uint4* z = reinterpret_cast<uint4*>(hist_smem);
      const int words = int(HistSmem<MODE>::kBytes / 16);
      for (int i = tid; i < words; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();

    const int ntiles = int((row_count + TILE - 1) / TILE);
    uint32_t r_next = (uint32_t(tid) < row_count) ? __ldg(rows + tid) : 0u;
    for (int t = 0; t < ntiles + NSTAGE - 1; ++t) {
      if (t < ntiles) {
        const int s = t % NSTAGE;
        const uint32_t pos = uint32_t(t) * TILE + tid;
        const uint32_t r = r_next < n ? r_next : 0u;  // row ids are < n by construction
        const uint32_t pos_next = pos + TILE;
        r_next = (pos_next < row_count) ? __ldg(rows + pos_next) : 0u;
        if (pos < row_count) {
          const uint8_t* src = bins + size_t(r) * kBlockFeatures;
          cp_async16(&stage_bins[(s * TILE + tid) * 2 + 0], src);
          cp_async16(&stage_bins[(s * TILE + tid) * 2 + 1], src + 16);
          cp_async8(&stage_gh[s * TILE + tid], gh + r);
        }
      }
      cp_async_commit();
      if (t >= NSTAGE - 1) {
        cp_async_wait<NSTAGE - 1>();
        __syncthreads();
        const int ct = t - (NSTAGE - 1);
        const int s = ct % NSTAGE;
        const int tile_rows = min(TILE, int(row_count) - ct * TILE);
#pragma unroll 1
        for (int step = 0; step < TILE / ROWS_PER_STEP; ++step) {
          const int rl = step * ROWS_PER_STEP + warp * 16 + int(r16);
          if (rl < tile_rows) {
            const uint4 v = rotate_bytes(stage_bins[(s * TILE + rl) * 2 + half], r16);
            const float2 p = stage_gh[s * TILE + rl];
            const uint32_t words[4] = {v.x, v.y, v.z, v.w};
            if constexpr (MODE == kModeFixed) {
              unsigned long long* hg = reinterpret_cast<unsigned long long*>(hist_smem);
              unsigned long long* hhc = hg + CELLS;
              const unsigned long long qg = (unsigned long long)quantize_f32(p.x, kg);
              const unsigned long long qhc =
                  (unsigned long long)quantize_f32(p.y, kh) + (1ull << kCountShift);
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const uint32_t b = (words[j >> 2] >> ((j & 3) * 8)) & 0xFFu;
                const uint32_t f = half * 16u + ((r16 + uint32_t(j)) & 15u);
                const uint32_t idx = b * kBlockFeatures + f;
                atomicAdd(&hg[idx], qg);
                atomicAdd(&hhc[idx], qhc);
              }
            } else {
              uint32_t* hc = reinterpret_cast<uint32_t*>(hist_smem);
              float* hgf = reinterpret_cast<float*>(hc + CELLS);
              float* hhf = hgf + CELLS;
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const uint32_t b = (words[j >> 2] >> ((j & 3) * 8)) & 0xFFu;
                const uint32_t f = half * 16u + ((r16 + uint32_t(j)) & 15u);
                const uint32_t idx = b * kBlockFeatures + f;
                atomicAdd(&hc[idx], 1u);
                atomicAdd(&hgf[idx], p.x);
                atomicAdd(&hhf[idx], p.y);
              }
            }
          }
        }
        __syncthreads();
      }
    }

    // Flush non-empty cells into the node's slot.
    unsigned long long* dst_base =
        a.hist + (size_t(e.slot) * a.features + size_t(fb) * kBlockFeatures) * kSlots * 3;
    for (int idx = tid; idx < CELLS; idx += THREADS) {
      const uint32_t b = idx / kBlockFeatures, f = idx % kBlockFeatures;
      if (fb * kBlockFeatures + f >= a.features) continue;
      unsigned long long* dst = dst_base + (size_t(f) * kSlots + b) * 3;
      if constexpr (MODE == kModeFixed) {
        const unsigned long long* hg = reinterpret_cast<const unsigned long long*>(hist_smem);
        const unsigned long long hcw = hg[CELLS + idx];
        const unsigned long long cnt = hcw >> kCountShift;
        if (cnt == 0) continue;
        atomicAdd(dst + 0, cnt);
        atomicAdd(dst + 1, hg[idx]);
        atomicAdd(dst + 2, hcw & ((1ull << kCountShift) - 1ull));
      } else {
        const uint32_t* hc = reinterpret_cast<const uint32_t*>(hist_smem);
        const float* hgf = reinterpret_cast<const float*>(hc + CELLS);
        const uint32_t cnt = hc[idx];
        if (cnt == 0) continue;
        atomicAdd(dst + 0, (unsigned long long)cnt);
        atomicAdd(reinterpret_cast<double*>(dst + 1), double(hgf[idx]));
        atomicAdd(reinterpret_cast<double*>(dst + 2), double(hgf[CELLS + idx]));
      }
    }
    if (tid == 0) {
      const uint32_t width = min(uint32_t(kBlockFeatures), a.features - fb * kBlockFeatures);
      atomicAdd(&a.ctl->cells, (unsigned long long)row_count * width);
      if (fb == 0) atomicAdd(&a.ctl->rows_built, (unsigned long long)row_count);
    }
    __syncthreads();
  }
}

template <int MODE, int THREADS, int NSTAGE>
size_t hist_smem_bytes() {
  return HistSmem<MODE>::kBytes + size_t(NSTAGE) * THREADS * (32 + 8);
}

template <int MODE, int THREADS, int NSTAGE>
cudaError_t launch_variant(const TrainerDev& a, int grid, cudaStream_t stream) {
  const size_t smem = hist_smem_bytes<MODE, THREADS, NSTAGE>();
  static bool configured = false;  // per variant; the attribute is per function
  if (!configured) {
    const cudaError_t err = cudaFuncSetAttribute(hist_build_kernel<MODE, THREADS, NSTAGE>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 int(smem));
    if (err != cudaSuccess) return err;
    configured = true;
  }
  hist_build_kernel<MODE, THREADS, NSTAGE><<<grid, THREADS, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_hist_build(const TrainerDev& a, const HistConfig& cfg, int grid,
                              cudaStream_t stream) {
  if (a.mode == kModeFixed) {
    if (cfg.threads == 1024) return launch_variant<kModeFixed, 1024, 2>(a, grid, stream);
    if (cfg.stages == 4) return launch_variant<kModeFixed, 512, 4>(a, grid, stream);
    if (cfg.stages == 2) return launch_variant<kModeFixed, 512, 2>(a, grid, stream);
    return launch_variant<kModeFixed, 512, 3>(a, grid, stream);
  }
  if (cfg.threads == 1024) return launch_variant<kModeFloat, 1024, 2>(a, grid, stream);
  if (cfg.stages == 4) return launch_variant<kModeFloat, 512, 4>(a, grid, stream);
  if (cfg.stages == 2) return launch_variant<kModeFloat, 512, 2>(a, grid, stream);
  return launch_variant<kModeFloat, 512, 3>(a, grid, stream);
}

}  // namespace mpsb
