// Histogram build for sm_103a: the hot kernel of the training path.
//
// Replaces the two-stage Metal histogram (src/mps/kernels/histogram.metal:34-182 driven
// by src/mps/mps_histogram.mm:82-256). Design:
//  * Bins are u8 rows padded to a multiple of 32 features; a work item reads its 32-byte
//    feature block of each gathered row with two 16-byte cp.async copies. The CTAs of the
//    4 feature blocks of a row chunk run together, so one HBM fetch of a row's line
//    serves all of them through L2. g/h arrive in the node's row order (the partition
//    moves them along with the row ids), so they stream instead of being gathered.
//  * Persistent CTAs (one per SM) pull work items (build node, row chunk <= 65536 rows,
//    feature block) from a device counter; every frontier node of every tree of a level
//    is in the same launch.
//  * A multi-stage cp.async pipeline stages each gathered row's 32-byte bin sector; the
//    staging thread also writes the row's quantized g/h (computed once per row) next to
//    it. Row ids are prefetched two tiles ahead and g/h one tile ahead in registers.
//  * The CTA-private histogram lives in shared memory laid out [bin][feature]. A warp
//    takes four staged rows at a time: each lane loads one 4-byte word (four features of
//    one row) and the row's values, then issues four rounds of reductions in which the
//    32 lanes touch 32 different features, so their words fall in different banks for
//    any bin values. Per four rows: one bins wavefront, one values wavefront, and one
//    red.shared per accumulator per feature.
//  * Only 32-bit integer shared reductions are native on sm_103 (64-bit and FP32 ones run
//    several times slower), so fixed mode splits each quantized value q (|q| <= 2^30) into
//    a 16-bit unsigned low limb and a signed high limb and accumulates count, g_lo, g_hi,
//    h_lo, h_hi as five u32 red.shared per cell. Over <= 2^16 rows no limb sum leaves 32
//    bits, so the int64 sum hi * 2^16 + lo is exact and order-independent. Float mode
//    (the plain path): a u32 count and two FP32 reductions per cell.
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
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

template <uint32_t OFF = 0>
__device__ __forceinline__ void red_shared_u32(uint32_t addr, uint32_t v) {
  asm volatile("red.shared.add.u32 [%0+%2], %1;\n" ::"r"(addr), "r"(v), "n"(OFF));
}
template <uint32_t OFF = 0>
__device__ __forceinline__ void red_shared_f32(uint32_t addr, float v) {
  asm volatile("red.shared.add.f32 [%0+%2], %1;\n" ::"r"(addr), "f"(v), "n"(OFF));
}

template <int MODE>
struct HistSmem;

template <>
struct HistSmem<kModeFixed> {  // count, g_lo, g_hi, h_lo, h_hi: five u32 words per cell
  static constexpr size_t kBytes = 5ull * kSlots * kBlockFeatures * sizeof(uint32_t);
};
template <>
struct HistSmem<kModeFixedG> {  // g_lo, g_hi
  static constexpr size_t kBytes = 2ull * kSlots * kBlockFeatures * sizeof(uint32_t);
};
template <>
struct HistSmem<kModeFloat> {
  static constexpr size_t kBytes = 3ull * kSlots * kBlockFeatures * sizeof(uint32_t);
};

// Per staged row: 32 bin bytes (cp.async) and 8 bytes of per-row values written by the
// staging thread: fixed mode the limbs {g_lo | h_lo << 16, g_hi | h_hi << 16} (16-bit
// each), gradient-only mode {g_lo | g_hi << 16, 0}, float mode {g, h}.
constexpr int kRowBytes = 32 + 8;

template <int MODE, int THREADS, int NSTAGE>
__global__ void __launch_bounds__(THREADS, 1) hist_build_kernel(TrainerDev a) {
  constexpr int WARPS = THREADS / 32;
  constexpr int CELLS = kSlots * kBlockFeatures;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* hist_smem = smem;
  uint8_t* stage_bins = smem + HistSmem<MODE>::kBytes;  // [WARPS][NSTAGE][32 rows][32]
  uint2* stage_val = reinterpret_cast<uint2*>(stage_bins + size_t(NSTAGE) * THREADS * 32);  // [WARPS][NSTAGE][32]

  __shared__ uint32_t s_item, s_entry;

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t n = a.n_rows;
  const uint32_t nfb = a.nfb;
  const uint32_t hist_base = static_cast<uint32_t>(__cvta_generic_to_shared(hist_smem));

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
    const uint32_t item_rows = a.item_rows ? a.item_rows : a.ctl->item_rows;
    const uint32_t row_begin = (chunk - a.build_prefix[s_entry]) * item_rows;
    const uint32_t row_count = row_begin < e.seg_cnt ? min(item_rows, e.seg_cnt - row_begin) : 0u;
    const size_t seg = (size_t(e.tree) * 2 + e.parity) * a.seg_stride + e.seg_off + row_begin;
    const uint32_t* rows = a.rows + seg;
    // g/h in segment order (contiguous) or by row id (gathered).
    const float2* gh_seg = a.gh_ordered ? a.gh + seg : nullptr;
    const float2* gh_row = a.gh_ordered ? nullptr : a.gh + size_t(e.tree) * n;
    const uint8_t* bins = a.bins + size_t(fb) * a.bins_block_stride;
    const int kg = a.trees[e.tree].kg;
    const int kh = a.trees[e.tree].kh;

    // Zero the CTA histogram.
    {
      uint4* z = reinterpret_cast<uint4*>(hist_smem);
      const int words = int(HistSmem<MODE>::kBytes / 16);
      for (int i = tid; i < words; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();

    // Each warp runs its own two-stage pipeline over 32-row tiles (tiles warp, warp +
    // WARPS, ...): lane l stages row l's quantized values by a shared store, and lanes 2j,
    // 2j+1 copy the two 16-byte halves of a row's 32-byte bin block with cp.async, while
    // the warp reduces the previous tile. Only
    // __syncwarp orders a warp's stages, so warps drift freely and keep the shared-memory
    // reduction pipe busy; the CTA meets only at item boundaries.
    const uint32_t ntiles = (row_count + 31u) / 32u;
    const uint32_t my_tiles = uint32_t(warp) < ntiles ? (ntiles - uint32_t(warp) + WARPS - 1) / WARPS : 0u;
    uint8_t* wbins = stage_bins + size_t(warp) * NSTAGE * 32 * 32;        // [NSTAGE][32][32]
    uint2* wval = stage_val + size_t(warp) * NSTAGE * 32;                  // [NSTAGE][32]
    // Register pipeline: row ids two tiles ahead, g/h one tile ahead.
    auto pos_of = [&](uint32_t k) -> uint32_t { return (uint32_t(warp) + k * WARPS) * 32u + uint32_t(lane); };
    auto row_at = [&](uint32_t pos) -> uint32_t {
      if (pos >= row_count) return 0u;
      const uint32_t r = __ldg(rows + pos);
      return r < n ? r : 0u;  // row ids are < n by construction
    };
    auto gh_at = [&](uint32_t pos, uint32_t r) -> float2 {
      if (pos >= row_count) return make_float2(0.f, 0.f);
      return gh_seg ? __ldg(gh_seg + pos) : __ldg(gh_row + r);
    };
    uint32_t r_cur = my_tiles > 0 ? row_at(pos_of(0)) : 0u;
    uint32_t r_nxt = my_tiles > 1 ? row_at(pos_of(1)) : 0u;
    float2 g_cur = my_tiles > 0 ? gh_at(pos_of(0), r_cur) : make_float2(0.f, 0.f);
    const uint32_t quad_byte = uint32_t(lane & 7) * 4u;
    const uint32_t rot = uint32_t(lane >> 3);
    // A warp takes a tile's rows four at a time: lane l reads the 4-byte word (l & 7) of
    // row l >> 3 (four features' bins) and that row's values, so one 128-byte wavefront
    // brings the bins of four rows and one more their values. In the i-th reduction round
    // lane l updates byte (i + (l >> 3)) & 3 of its word: across the warp the 32 features
    // are distinct, so the 32 words fall in 32 different banks.
    auto accumulate = [&](uint32_t f, uint32_t b, uint2 q) {
      const uint32_t addr = hist_base + (b * kBlockFeatures + f) * 4u;
      if constexpr (MODE == kModeFixed) {
        red_shared_u32<0>(addr, 1u);
        red_shared_u32<1u * CELLS * 4u>(addr, q.x & 0xFFFFu);
        red_shared_u32<2u * CELLS * 4u>(addr, uint32_t(int32_t(int16_t(q.y & 0xFFFFu))));
        red_shared_u32<3u * CELLS * 4u>(addr, q.x >> 16);
        red_shared_u32<4u * CELLS * 4u>(addr, q.y >> 16);
      } else if constexpr (MODE == kModeFixedG) {
        red_shared_u32<0>(addr, q.x & 0xFFFFu);
        red_shared_u32<1u * CELLS * 4u>(addr, uint32_t(int32_t(q.x) >> 16));
      } else {
        red_shared_u32<0>(addr, 1u);
        red_shared_f32<CELLS * 4u>(addr, __uint_as_float(q.x));
        red_shared_f32<2u * CELLS * 4u>(addr, __uint_as_float(q.y));
      }
    };
    for (uint32_t k = 0; k < my_tiles + 1; ++k) {
      if (k < my_tiles) {
        const int st = int(k % NSTAGE);
        const uint32_t pos = pos_of(k);
        const uint32_t r = r_cur;
        const float2 p = g_cur;
        const uint32_t r_far = k + 2 < my_tiles ? row_at(pos_of(k + 2)) : 0u;
        g_cur = k + 1 < my_tiles ? gh_at(pos_of(k + 1), r_nxt) : make_float2(0.f, 0.f);
        r_cur = r_nxt;
        r_nxt = r_far;
        // Two lanes per row: each copy instruction touches 16 rows' lines instead of 32.
        const uint32_t valid = min(32u, row_count - (uint32_t(warp) + k * WARPS) * 32u);
#pragma unroll
        for (uint32_t i = 0; i < 2; ++i) {
          const uint32_t row_in_tile = 16u * i + uint32_t(lane >> 1);
          const uint32_t rr = __shfl_sync(0xffffffffu, r, int(row_in_tile));
          const uint32_t half = uint32_t(lane & 1) * 16u;
          if (row_in_tile < valid)
            cp_async16(wbins + (size_t(st) * 32 + row_in_tile) * 32 + half,
                       bins + size_t(rr) * a.bins_row_stride + half);
        }
        if (pos < row_count) {
          uint2 v;
          if constexpr (MODE == kModeFixed) {
            // |q| <= 2^30: low limb = q & 0xFFFF (unsigned), high limb = q >> 16 (signed,
            // |hi| <= 2^14 fits in 16 bits).
            const long long qg = quantize_f32(p.x, kg);
            const long long qh = quantize_f32(p.y, kh);
            const uint32_t glo = uint32_t(qg) & 0xFFFFu, ghi = uint32_t(qg >> 16) & 0xFFFFu;
            const uint32_t hlo = uint32_t(qh) & 0xFFFFu, hhi = uint32_t(qh >> 16) & 0xFFFFu;
            v = make_uint2(glo | (hlo << 16), ghi | (hhi << 16));
          } else if constexpr (MODE == kModeFixedG) {
            // |q| <= 2^30: the low 32 bits hold q in two's complement; the reductions
            // take its unsigned low and signed high 16 bits.
            v = make_uint2(uint32_t(quantize_f32(p.x, kg)), 0u);
          } else {
            v = make_uint2(__float_as_uint(p.x), __float_as_uint(p.y));
          }
          wval[st * 32 + lane] = v;
        }
      }
      cp_async_commit();
      if (k >= 1) {
        cp_async_wait<1>();
        __syncwarp();
        const uint32_t ct = k - 1;
        const int st = int(ct % NSTAGE);
        const uint32_t tile_pos = (uint32_t(warp) + ct * WARPS) * 32u;
        const int nrows = int(min(32u, row_count - tile_pos));
        const uint8_t* sb = wbins + size_t(st) * 32 * 32;
        const uint2* sv = wval + st * 32;
        for (int j = 0; j < nrows; j += 4) {
          const int r = j + int(rot);
          if (r < nrows) {
            const uint32_t w = *reinterpret_cast<const uint32_t*>(sb + r * 32 + quad_byte);
            const uint2 q = sv[r];
#pragma unroll
            for (uint32_t i = 0; i < 4; ++i) {
              const uint32_t sel = (i + rot) & 3u;
              accumulate(quad_byte + sel, (w >> (8u * sel)) & 0xFFu, q);
            }
          }
        }
        __syncwarp();
      }
    }
    cp_async_wait<0>();
    __syncthreads();

    // Flush non-empty cells into the node's slot.
    unsigned long long* dst_base =
        a.hist + (size_t(e.slot) * a.features + size_t(fb) * kBlockFeatures) * kSlots * 3;
    for (int idx = tid; idx < CELLS; idx += THREADS) {
      const uint32_t b = idx / kBlockFeatures, f = idx % kBlockFeatures;
      if (fb * kBlockFeatures + f >= a.features) continue;
      unsigned long long* dst = dst_base + (size_t(f) * kSlots + b) * 3;
      if constexpr (MODE == kModeFixed) {
        const uint32_t* w = reinterpret_cast<const uint32_t*>(hist_smem);
        const uint32_t cnt = w[idx];
        if (cnt == 0) continue;
        const long long g = (long long)int32_t(w[2 * CELLS + idx]) * 65536 + (long long)w[CELLS + idx];
        const long long hh = (long long)w[4 * CELLS + idx] * 65536 + (long long)w[3 * CELLS + idx];
        atomicAdd(dst + 0, (unsigned long long)cnt);
        atomicAdd(dst + 1, (unsigned long long)g);
        atomicAdd(dst + 2, (unsigned long long)hh);
      } else if constexpr (MODE == kModeFixedG) {
        const uint32_t* w = reinterpret_cast<const uint32_t*>(hist_smem);
        const long long g = (long long)int32_t(w[CELLS + idx]) * 65536 + (long long)w[idx];
        if (g != 0) atomicAdd(dst + 1, (unsigned long long)g);
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
  return HistSmem<MODE>::kBytes + size_t(NSTAGE) * THREADS * kRowBytes;
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
  // Shared memory: 160 KB (fixed) / 64 KB (gradient only) / 96 KB (float) histogram +
  // stages x threads x 40 B.
  if (a.mode == kModeFixedG) {
    if (cfg.root_threads == 1024) return launch_variant<kModeFixedG, 1024, 2>(a, grid, stream);
    return launch_variant<kModeFixedG, 768, 2>(a, grid, stream);
  }
  if (a.mode == kModeFixed) {
    if (cfg.threads == 768) return launch_variant<kModeFixed, 768, 2>(a, grid, stream);
    if (cfg.threads == 640) return launch_variant<kModeFixed, 640, 2>(a, grid, stream);
    if (cfg.stages == 2) return launch_variant<kModeFixed, 512, 2>(a, grid, stream);
    return launch_variant<kModeFixed, 512, 3>(a, grid, stream);
  }
  if (cfg.threads == 1024) return launch_variant<kModeFloat, 1024, 2>(a, grid, stream);
  if (cfg.threads == 768) return launch_variant<kModeFloat, 768, 2>(a, grid, stream);
  if (cfg.stages == 2) return launch_variant<kModeFloat, 512, 2>(a, grid, stream);
  return launch_variant<kModeFloat, 512, 3>(a, grid, stream);
}

}  // namespace mpsb
