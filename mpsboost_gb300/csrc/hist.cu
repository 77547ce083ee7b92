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
//  * Datasets with more than 256 histogram slots per feature (u16 bins) build with
//    hist_build_wide_kernel, at the end of this file.
#include <algorithm>
#include <type_traits>

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

// ---- TMA gather4 staging (row-major levels) ------------------------------------------
// A warp's stage is filled by up to eight `cp.async.bulk.tensor.2d ... tile::gather4`
// copies (four 32-byte rows each, 128 bytes into a 128-byte aligned slot) that complete
// on the stage's mbarrier. The L1 tag stage sees none of it (the cp.async path costs one
// L1 wavefront per gathered row's line), but on GB300 the copies complete later than
// cp.async ones and the row-major levels build about 8 % slower, so this path is opt-in.
constexpr unsigned long long kCopyTimeoutNs = 1000000000ull;  // 1 s per stage wait

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}
// The waiting thread sleeps until the phase completes or 20 us pass (no spinning issue
// slots or shared-memory requests while the copies are in flight).
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 20000;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Waits for the phase of the given parity to complete; false after kCopyTimeoutNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kCopyTimeoutNs) return false;
  }
}
__device__ __forceinline__ void tma_gather4(uint32_t dst, const CUtensorMap* map, int32_t x,
                                            int32_t r0, int32_t r1, int32_t r2, int32_t r3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(bar)
      : "memory");
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
struct HistSmem<kModeFixedCG> {  // count, g_lo, g_hi
  static constexpr size_t kBytes = 3ull * kSlots * kBlockFeatures * sizeof(uint32_t);
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

// TMA: stage gathered rows with tile::gather4 copies through `tmap` (row-major bins);
// otherwise with cp.async (either layout; `tmap` unused).
template <int MODE, int THREADS, int NSTAGE, bool TMA>
__global__ void __launch_bounds__(THREADS, 1)
    hist_build_kernel(TrainerDev a, const __grid_constant__ CUtensorMap tmap) {
  constexpr int WARPS = THREADS / 32;
  constexpr int CELLS = kSlots * kBlockFeatures;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* hist_smem = smem;
  uint8_t* stage_bins = smem + HistSmem<MODE>::kBytes;  // [WARPS][NSTAGE][32 rows][32]
  uint2* stage_val = reinterpret_cast<uint2*>(stage_bins + size_t(NSTAGE) * THREADS * 32);  // [WARPS][NSTAGE][32]
  // TMA: one mbarrier per warp and stage, [WARPS][NSTAGE].
  const uint32_t bar_base =
      static_cast<uint32_t>(__cvta_generic_to_shared(stage_val + size_t(NSTAGE) * THREADS));

  __shared__ uint32_t s_item, s_entry, s_abort;

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t n = a.n_rows;
  const uint32_t nfb = a.nfb;
  const uint32_t hist_base = static_cast<uint32_t>(__cvta_generic_to_shared(hist_smem));
  const uint32_t stage_base = static_cast<uint32_t>(__cvta_generic_to_shared(stage_bins));

  if constexpr (TMA) {
    // gather4 writes 128-byte slots; the staging area starts 128-byte aligned.
    if (stage_base & 127u) {
      if (tid == 0) atomicOr(&a.ctl->error, uint32_t(kErrCopy));
      return;
    }
    if (lane == 0)
      for (int st = 0; st < NSTAGE; ++st) mbar_init(bar_base + uint32_t(warp * NSTAGE + st) * 8u, 1u);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (tid == 0) s_abort = 0;
  __syncthreads();
  uint32_t warp_tiles = 0;  // tiles this warp staged so far (stage and mbarrier phase)

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
    if (item >= limit || s_abort) break;
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
    // Unit-hessian builds: the quantized hessian of every row, round_half_even(2^kh).
    const long long q_unit_h = MODE == kModeFixedCG ? quantize_f32(1.0f, kh) : 0ll;

    // Zero the CTA histogram.
    {
      uint4* z = reinterpret_cast<uint4*>(hist_smem);
      const int words = int(HistSmem<MODE>::kBytes / 16);
      for (int i = tid; i < words; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();

    // Each warp runs its own NSTAGE-stage pipeline over 32-row tiles (tiles warp, warp +
    // WARPS, ...): lane l stages row l's quantized values by a shared store, and lanes 2j,
    // 2j+1 copy the two 16-byte halves of a row's 32-byte bin block with cp.async (or
    // lane 4j gathers four rows with TMA), while the warp reduces the tile NSTAGE - 1
    // back. Only __syncwarp orders a warp's stages, so warps drift freely and keep the
    // shared-memory reduction pipe busy; the CTA meets only at item boundaries.
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
      } else if constexpr (MODE == kModeFixedCG) {
        red_shared_u32<0>(addr, 1u);
        red_shared_u32<1u * CELLS * 4u>(addr, q.x & 0xFFFFu);
        red_shared_u32<2u * CELLS * 4u>(addr, uint32_t(int32_t(q.x) >> 16));
      } else {
        red_shared_u32<0>(addr, 1u);
        red_shared_f32<CELLS * 4u>(addr, __uint_as_float(q.x));
        red_shared_f32<2u * CELLS * 4u>(addr, __uint_as_float(q.y));
      }
    };
    // Iteration k stages tile k and reduces tile k - AHEAD.
    constexpr uint32_t AHEAD = NSTAGE - 1;
    for (uint32_t k = 0; k < my_tiles + AHEAD; ++k) {
      if (k < my_tiles) {
        const int st = int((warp_tiles + k) % NSTAGE);
        const uint32_t pos = pos_of(k);
        const uint32_t r = r_cur;
        const float2 p = g_cur;
        const uint32_t r_far = k + 2 < my_tiles ? row_at(pos_of(k + 2)) : 0u;
        g_cur = k + 1 < my_tiles ? gh_at(pos_of(k + 1), r_nxt) : make_float2(0.f, 0.f);
        r_cur = r_nxt;
        r_nxt = r_far;
        const uint32_t valid = min(32u, row_count - (uint32_t(warp) + k * WARPS) * 32u);
        if constexpr (TMA) {
          // Lane 4j gathers rows 4j..4j+3 of the tile into slot j; positions past the
          // tile's end carry row 0, so every coordinate is a row of the matrix.
          const int quad = lane & ~3;
          const uint32_t r1 = __shfl_sync(0xffffffffu, r, quad + 1);
          const uint32_t r2 = __shfl_sync(0xffffffffu, r, quad + 2);
          const uint32_t r3 = __shfl_sync(0xffffffffu, r, quad + 3);
          const uint32_t groups = (valid + 3u) / 4u;
          const uint32_t bar = bar_base + uint32_t(warp * NSTAGE + st) * 8u;
          if (lane == 0) mbar_arrive_expect_tx(bar, groups * 128u);
          __syncwarp();
          // The slot's previous contents were read by the reduction NSTAGE tiles back,
          // whose loaded words fed its reductions before the __syncwarp that ended it:
          // those reads are complete, so the async-proxy write needs no proxy fence.
          if ((lane & 3) == 0 && uint32_t(lane >> 2) < groups) {
            tma_gather4(stage_base + uint32_t((warp * NSTAGE + st) * 32 + lane) * 32u, &tmap,
                        int32_t(fb * kBlockFeatures), int32_t(r), int32_t(r1), int32_t(r2),
                        int32_t(r3), bar);
          }
        } else {
          // Two lanes per row: each copy instruction touches 16 rows' lines instead of 32.
#pragma unroll
          for (uint32_t i = 0; i < 2; ++i) {
            const uint32_t row_in_tile = 16u * i + uint32_t(lane >> 1);
            const uint32_t rr = __shfl_sync(0xffffffffu, r, int(row_in_tile));
            const uint32_t half = uint32_t(lane & 1) * 16u;
            if (row_in_tile < valid)
              cp_async16(wbins + (size_t(st) * 32 + row_in_tile) * 32 + half,
                         bins + size_t(rr) * a.bins_row_stride + half);
          }
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
          } else if constexpr (MODE == kModeFixedG || MODE == kModeFixedCG) {
            // |q| <= 2^30: the low 32 bits hold q in two's complement; the reductions
            // take its unsigned low and signed high 16 bits.
            v = make_uint2(uint32_t(quantize_f32(p.x, kg)), 0u);
          } else {
            v = make_uint2(__float_as_uint(p.x), __float_as_uint(p.y));
          }
          wval[st * 32 + lane] = v;
        }
      }
      if constexpr (!TMA) cp_async_commit();
      if (k >= AHEAD) {
        const uint32_t ct = k - AHEAD;
        const int st = int((warp_tiles + ct) % NSTAGE);
        if constexpr (TMA) {
          const uint32_t phase = ((warp_tiles + ct) / NSTAGE) & 1u;
          const bool ok = __all_sync(0xffffffffu,
                                     mbar_wait_bounded(bar_base + uint32_t(warp * NSTAGE + st) * 8u, phase));
          if (!ok) {
            // Wait (bounded) for the later tiles' copies, already issued, then give up
            // the launch: the host sees kErrCopy and discards the round.
            for (uint32_t t = ct + 1; t <= k && t < my_tiles; ++t) {
              const uint32_t nt = warp_tiles + t;
              mbar_wait_bounded(bar_base + uint32_t(warp * NSTAGE + int(nt % NSTAGE)) * 8u,
                                (nt / NSTAGE) & 1u);
            }
            if (lane == 0) {
              atomicOr(&a.ctl->error, uint32_t(kErrCopy));
              *reinterpret_cast<volatile uint32_t*>(&s_abort) = 1u;
            }
            break;
          }
        } else {
          cp_async_wait<AHEAD>();
        }
        __syncwarp();
        const uint32_t tile_pos = (uint32_t(warp) + ct * WARPS) * 32u;
        const int nrows = int(min(32u, row_count - tile_pos));
        const uint8_t* sb = wbins + size_t(st) * 32 * 32;
        const uint2* sv = wval + st * 32;
        auto reduce_rows = [&](int r) {
          const uint32_t w = *reinterpret_cast<const uint32_t*>(sb + r * 32 + quad_byte);
          const uint2 q = sv[r];
#pragma unroll
          for (uint32_t i = 0; i < 4; ++i) {
            const uint32_t sel = (i + rot) & 3u;
            accumulate(quad_byte + sel, __byte_perm(w, 0u, 0x4440u | sel), q);  // byte sel of w
          }
        };
        if (nrows == 32) {  // full tile: no bounds tests, the eight groups unrolled
#pragma unroll
          for (int j = 0; j < 32; j += 4) reduce_rows(j + int(rot));
        } else {
          for (int j = 0; j < nrows; j += 4) {
            const int r = j + int(rot);
            if (r < nrows) reduce_rows(r);
          }
        }
        __syncwarp();
      }
    }
    warp_tiles += my_tiles;
    if constexpr (!TMA) cp_async_wait<0>();
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
      } else if constexpr (MODE == kModeFixedCG) {
        const uint32_t* w = reinterpret_cast<const uint32_t*>(hist_smem);
        const uint32_t cnt = w[idx];
        if (cnt == 0) continue;
        const long long g = (long long)int32_t(w[2 * CELLS + idx]) * 65536 + (long long)w[CELLS + idx];
        atomicAdd(dst + 0, (unsigned long long)cnt);
        atomicAdd(dst + 1, (unsigned long long)g);
        atomicAdd(dst + 2, (unsigned long long)((long long)cnt * q_unit_h));
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

template <int MODE, int THREADS, int NSTAGE, bool TMA>
size_t hist_smem_bytes() {
  return HistSmem<MODE>::kBytes + size_t(NSTAGE) * THREADS * kRowBytes +
         (TMA ? size_t(THREADS / 32) * NSTAGE * 8 : 0);
}

// ---- Register-direct variant (fixed-point modes) ---------------------------------------
//
// Measured on GB300 (ncu, 4M x 128): the staged kernels keep the L1 data pipe (one
// wavefront per clock per SM, shared by shared-memory reductions and global-load data)
// 75-85 % busy, spending per gathered 32-byte row block 5 wavefronts on reductions, about 1
// on the staged bins and values and about 2 on the two 16-byte cp.async copies; and each
// work item's flush (3 x 8192 single-word red.global, each warp instruction touching 32
// lines) made small items expensive. This variant loads each row's block with one
// 256-bit load into registers, reduces straight from registers, and flushes through TMA
// bulk reductions.

struct Bins32 {
  uint32_t w[8];
};
// One 32-byte load (a row's feature block) into registers, without L1 allocation.
__device__ __forceinline__ Bins32 ld_nc_na_v8(const void* p) {
  Bins32 v;
  asm volatile("ld.global.nc.L1::no_allocate.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
               : "=r"(v.w[0]), "=r"(v.w[1]), "=r"(v.w[2]), "=r"(v.w[3]), "=r"(v.w[4]), "=r"(v.w[5]),
                 "=r"(v.w[6]), "=r"(v.w[7])
               : "l"(p));
  return v;
}

// Flush through TMA bulk reductions, for kernels with kFlushBytes of free shared memory at
// `staging`. The CTA histogram is bin-major ([bin][feature], so that the reductions of a
// warp hit 32 banks) and the node's slot feature-major ([feature][bin] {count, g, h}).
// Each of kFlushWarps warps takes tiles of 32 features x 8 bins: lane f reads its
// feature's 8 cells (conflict-free), writes their 24 words into its row of the warp's
// staging tile in the slot's order, and hands the row to one 192-byte
// `cp.reduce.async.bulk ... .add.u64`, which L2 applies a sector at a time instead of as
// 24 single-word atomics. All-zero rows are skipped. Every thread of the CTA calls it.
constexpr int kFlushWarps = 8;
constexpr int kFlushBins = 8;
constexpr int kFlushRowWords = kFlushBins * 3 + 2;  // a feature's 24 words, padded to 16 bytes
constexpr size_t kFlushBytes = size_t(kFlushWarps) * kBlockFeatures * kFlushRowWords * 8;

__device__ __forceinline__ void bulk_reduce_add_u64(void* gdst, uint32_t ssrc, uint32_t bytes) {
  asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.u64 [%0], [%1], %2;\n" ::"l"(gdst),
               "r"(ssrc), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// The shared source of this thread's bulk operations may be written again.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// This thread's bulk operations are complete (their global writes performed).
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

template <int MODE, int THREADS>
__device__ __forceinline__ void flush_cta_histogram_bulk(const TrainerDev& a, const BuildEntry& e, uint32_t fb,
                                                         const unsigned char* hist_smem,
                                                         unsigned long long* staging, long long q_unit_h,
                                                         uint32_t row_count) {
  static_assert(THREADS / 32 > kFlushWarps, "flush warps and a spare warp");
  constexpr int CELLS = kSlots * kBlockFeatures;
  const int tid = threadIdx.x;
  const uint32_t lane = uint32_t(tid & 31);
  const int warp = tid >> 5;
  const uint32_t width = min(uint32_t(kBlockFeatures), a.features - fb * kBlockFeatures);
  if (warp < kFlushWarps) {
    unsigned long long* dst_base =
        a.hist + (size_t(e.slot) * a.features + size_t(fb) * kBlockFeatures) * kSlots * 3;
    unsigned long long* row = staging + (size_t(warp) * kBlockFeatures + lane) * kFlushRowWords;
    const uint32_t row_addr = static_cast<uint32_t>(__cvta_generic_to_shared(row));
    const uint32_t* w = reinterpret_cast<const uint32_t*>(hist_smem);
    for (uint32_t grp = uint32_t(warp); grp < kSlots / kFlushBins; grp += kFlushWarps) {
      const uint32_t b0 = grp * kFlushBins;
      bulk_wait_read();  // the row's previous bulk reduction has read it
      unsigned long long any = 0;
#pragma unroll
      for (uint32_t j = 0; j < kFlushBins; ++j) {
        const uint32_t idx = (b0 + j) * kBlockFeatures + lane;
        unsigned long long c, g, h;
        if constexpr (MODE == kModeFixed) {
          c = w[idx];
          g = (unsigned long long)((long long)int32_t(w[2 * CELLS + idx]) * 65536 + (long long)w[CELLS + idx]);
          h = (unsigned long long)((long long)w[4 * CELLS + idx] * 65536 + (long long)w[3 * CELLS + idx]);
        } else if constexpr (MODE == kModeFixedG) {
          c = 0;  // the gradient-only root's count and hessian words are restored afterwards
          g = (unsigned long long)((long long)int32_t(w[CELLS + idx]) * 65536 + (long long)w[idx]);
          h = 0;
        } else {
          c = w[idx];
          g = (unsigned long long)((long long)int32_t(w[2 * CELLS + idx]) * 65536 + (long long)w[CELLS + idx]);
          h = (unsigned long long)((long long)c * q_unit_h);
        }
        row[3 * j + 0] = c;
        row[3 * j + 1] = g;
        row[3 * j + 2] = h;
        any |= c | g | h;
      }
      if (lane < width && any != 0ull) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the row's stores before the bulk read
        bulk_reduce_add_u64(dst_base + (size_t(lane) * kSlots + b0) * 3, row_addr, kFlushBins * 3 * 8);
        bulk_commit();
      }
    }
    bulk_wait_read();  // the staging rows are free for the next item
  }
  if (tid == 0) {
    atomicAdd(&a.ctl->cells, (unsigned long long)row_count * width);
    if (fb == 0) atomicAdd(&a.ctl->rows_built, (unsigned long long)row_count);
  }
}

// A work item's description, prepared one item ahead by one warp.
struct ItemDesc {
  uint32_t item, limit, fb, row_begin, row_count;
  int kg, kh;
  BuildEntry e;
};

// Takes the next work item from the device counter and describes it (one warp; lane 0
// writes *out). The build entry holding the item's row chunk is the last one whose chunk
// prefix is <= the chunk, found by a 32-way search of the prefix table.
__device__ __forceinline__ void fetch_item_warp(const TrainerDev& a, uint32_t lane, ItemDesc* out) {
  uint32_t item = 0;
  if (lane == 0) item = a.item_begin + atomicAdd(&a.ctl->hist_counter, 1u);
  item = __shfl_sync(0xffffffffu, item, 0);
  const uint32_t limit = a.item_end ? a.item_end : a.ctl->hist_items;
  ItemDesc d{};
  d.item = item;
  d.limit = limit;
  if (item < limit) {
    const uint32_t chunk = item / a.nfb;
    uint32_t lo = 0, hi = a.ctl->n_build;  // build_prefix[lo] <= chunk < build_prefix[hi]
    while (hi - lo > 1) {
      const uint32_t step = (hi - lo + 31) / 32;
      const uint32_t pos = lo + lane * step;
      const bool ok = pos < hi && a.build_prefix[pos] <= chunk;  // true on lane 0
      const uint32_t last = 31u - uint32_t(__clz(__ballot_sync(0xffffffffu, ok)));
      lo += last * step;
      hi = min(hi, lo + step);
    }
    d.e = a.build[lo];
    const uint32_t item_rows = a.item_rows ? a.item_rows : a.ctl->item_rows;
    d.fb = item % a.nfb;
    d.row_begin = (chunk - a.build_prefix[lo]) * item_rows;
    d.row_count = d.row_begin < d.e.seg_cnt ? min(item_rows, d.e.seg_cnt - d.row_begin) : 0u;
    d.kg = a.trees[d.e.tree].kg;
    d.kh = a.trees[d.e.tree].kh;
  }
  if (lane == 0) *out = d;
}

// The kernel. A warp takes its rows 32 at a time: lane l owns row l of the group, loads the
// row's whole 32-byte feature block with one 256-bit load and the row's g/h, which it
// quantizes once. In reduction round i (0..31) lane l updates feature i ^ l: for each i
// the 32 lanes touch 32 different features, hence 32 different banks. The row's 32 bytes
// are permuted once (words by l >> 2, bytes within a word by l & 3) so that round i reads
// the fixed byte i. Row ids are loaded three groups ahead, bins and g/h two ahead; the
// warps meet only at work-item boundaries (zero, flush), while warp kFlushWarps fetches the
// next item's description during the flush.
template <int MODE, int THREADS, int PF>
__global__ void __launch_bounds__(THREADS, 1) hist_build_direct_kernel(TrainerDev a) {
  static_assert(PF >= 2 && PF <= 4, "bins and pairs 2-4 groups ahead");
  static_assert(MODE == kModeFixed || MODE == kModeFixedCG || MODE == kModeFixedG, "fixed-point modes");
  static_assert(THREADS / 32 > kFlushWarps, "a warp besides the flush warps fetches the next item");
  constexpr int WARPS = THREADS / 32;
  constexpr int CELLS = kSlots * kBlockFeatures;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* hist_smem = smem;
  // The next item's description lives after the flush staging; with no static shared
  // memory the histogram starts the CTA's dynamic shared memory (128-byte aligned in
  // practice, which the reduction address arithmetic exploits; checked below).
  ItemDesc* s_desc = reinterpret_cast<ItemDesc*>(smem + HistSmem<MODE>::kBytes + kFlushBytes);

  const int tid = threadIdx.x;
  const uint32_t lane = uint32_t(tid & 31);
  const int warp = tid >> 5;
  const uint32_t n = a.n_rows;
  const uint32_t hist_base = static_cast<uint32_t>(__cvta_generic_to_shared(hist_smem));
  const uint32_t lw = lane >> 2;
  const uint32_t lb = lane & 3u;
  const uint32_t byte_sel = (0u ^ lb) | ((1u ^ lb) << 4) | ((2u ^ lb) << 8) | ((3u ^ lb) << 12);

  if (warp == kFlushWarps) fetch_item_warp(a, lane, s_desc);
  __syncthreads();
  // With hist_base 128-byte aligned, hist_base + 4 (lane ^ i) = (hist_base + 4 lane) ^ 4 i
  // (4 lane and 4 i stay below 128), one instruction per reduction round.
  const bool aligned = (hist_base & 127u) == 0u;  // CTA-uniform
  const uint32_t lane_base = hist_base + lane * 4u;
  for (;;) {
    const ItemDesc d = *s_desc;
    if (d.item >= d.limit) break;
    const uint32_t fb = d.fb;
    const BuildEntry e = d.e;
    const uint32_t row_count = d.row_count;
    const size_t seg = (size_t(e.tree) * 2 + e.parity) * a.seg_stride + e.seg_off + d.row_begin;
    const uint32_t* rows = a.rows + seg;
    const float2* gh_seg = a.gh_ordered ? a.gh + seg : nullptr;
    const float2* gh_row = a.gh_ordered ? nullptr : a.gh + size_t(e.tree) * n;
    const uint8_t* bins = a.bins + size_t(fb) * a.bins_block_stride;
    const uint64_t row_stride = a.bins_row_stride;
    const int kg = d.kg;
    const int kh = d.kh;
    const long long q_unit_h = MODE == kModeFixedCG ? quantize_f32(1.0f, kh) : 0ll;
    {
      uint4* z = reinterpret_cast<uint4*>(hist_smem);
      const int words = int(HistSmem<MODE>::kBytes / 16);
      for (int i = tid; i < words; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();  // also: every thread holds this item's description

    const uint32_t ngroups = (row_count + 31u) / 32u;
    const uint32_t my = uint32_t(warp) < ngroups ? (ngroups - uint32_t(warp) + WARPS - 1) / WARPS : 0u;
    auto pos_of = [&](uint32_t k) -> uint32_t { return (uint32_t(warp) + k * WARPS) * 32u + lane; };
    auto row_at = [&](uint32_t k) -> uint32_t {
      const uint32_t pos = pos_of(k);
      if (k >= my || pos >= row_count) return 0u;
      const uint32_t r = __ldg(rows + pos);
      return r < n ? r : 0u;  // row ids are < n by construction
    };
    auto bins_at = [&](uint32_t k, uint32_t r) -> Bins32 {
      if (k >= my) return Bins32{};
      return ld_nc_na_v8(bins + size_t(r) * row_stride);
    };
    auto gh_at = [&](uint32_t k, uint32_t r) -> float2 {
      const uint32_t pos = pos_of(k);
      if (k >= my || pos >= row_count) return make_float2(0.f, 0.f);
      return gh_seg ? __ldg(gh_seg + pos) : __ldg(gh_row + r);
    };
    // Ring of the next PF groups' bins and pairs; the row id of group k + PF is loaded
    // one iteration before its bins.
    Bins32 bq[PF];
    float2 gq[PF];
#pragma unroll
    for (int j = 0; j < PF; ++j) {
      const uint32_t r = row_at(uint32_t(j));
      bq[j] = bins_at(uint32_t(j), r);
      gq[j] = gh_at(uint32_t(j), r);
    }
    uint32_t r_ahead = row_at(PF);
    for (uint32_t k = 0; k < my; ++k) {
      const uint32_t r_next = row_at(k + PF + 1);
      const Bins32 b_new = bins_at(k + PF, r_ahead);
      const float2 g_new = gh_at(k + PF, r_ahead);
      const Bins32& b0 = bq[0];
      const float2& g0 = gq[0];
      if (pos_of(k) < row_count) {
        // Limbs of the row's quantized values (|q| <= 2^30): unsigned low 16 bits and the
        // signed high part.
        uint32_t glo, ghi, hlo = 0, hhi = 0;
        {
          const long long qg = quantize_f32(g0.x, kg);
          glo = uint32_t(qg) & 0xFFFFu;
          ghi = uint32_t(int32_t(qg >> 16));
          if constexpr (MODE == kModeFixed) {
            const long long qh = quantize_f32(g0.y, kh);
            hlo = uint32_t(qh) & 0xFFFFu;
            hhi = uint32_t(qh >> 16);
          }
        }
        // w[k] = word k ^ lw of the row's block with its bytes permuted by lb: byte i of w
        // is byte i ^ lane of the block (feature i ^ lane).
        uint32_t w[8];
#pragma unroll
        for (uint32_t k8 = 0; k8 < 8; ++k8) w[k8] = b0.w[k8];
#pragma unroll
        for (uint32_t bit = 1; bit < 8; bit <<= 1) {
          const bool swap = (lw & bit) != 0;  // per lane: selects, no divergence
#pragma unroll
          for (uint32_t k8 = 0; k8 < 8; ++k8)
            if ((k8 & bit) == 0) {
              const uint32_t x = w[k8], y = w[k8 | bit];
              w[k8] = swap ? y : x;
              w[k8 | bit] = swap ? x : y;
            }
        }
#pragma unroll
        for (uint32_t k8 = 0; k8 < 8; ++k8) w[k8] = __byte_perm(w[k8], 0u, byte_sel);
        auto reduce_row = [&](auto aligned_tag) {
          constexpr bool ALIGNED = decltype(aligned_tag)::value;
#pragma unroll
          for (uint32_t i = 0; i < 32; ++i) {
            const uint32_t bin = (w[i >> 2] >> (8u * (i & 3u))) & 0xFFu;
            const uint32_t cell = ALIGNED ? (lane_base ^ (i << 2)) : hist_base + ((lane ^ i) << 2);
            const uint32_t addr = cell + (bin << 7);  // bin * kBlockFeatures * 4 bytes
            if constexpr (MODE == kModeFixed) {
              red_shared_u32<0>(addr, 1u);
              red_shared_u32<1u * CELLS * 4u>(addr, glo);
              red_shared_u32<2u * CELLS * 4u>(addr, ghi);
              red_shared_u32<3u * CELLS * 4u>(addr, hlo);
              red_shared_u32<4u * CELLS * 4u>(addr, hhi);
            } else if constexpr (MODE == kModeFixedG) {
              red_shared_u32<0>(addr, glo);
              red_shared_u32<1u * CELLS * 4u>(addr, ghi);
            } else {
              red_shared_u32<0>(addr, 1u);
              red_shared_u32<1u * CELLS * 4u>(addr, glo);
              red_shared_u32<2u * CELLS * 4u>(addr, ghi);
            }
          }
        };
        if (aligned) reduce_row(std::true_type{});
        else reduce_row(std::false_type{});
      }
#pragma unroll
      for (int j = 0; j + 1 < PF; ++j) {
        bq[j] = bq[j + 1];
        gq[j] = gq[j + 1];
      }
      bq[PF - 1] = b_new;
      gq[PF - 1] = g_new;
      r_ahead = r_next;
    }
    __syncthreads();
    // The next item's description is fetched while the flush warps work.
    if (warp == kFlushWarps) fetch_item_warp(a, lane, s_desc);
    flush_cta_histogram_bulk<MODE, THREADS>(
        a, e, fb, hist_smem, reinterpret_cast<unsigned long long*>(hist_smem + HistSmem<MODE>::kBytes),
        q_unit_h, row_count);
    __syncthreads();
  }
  bulk_wait_all();  // this thread's bulk reductions have reached the slots
}

template <int MODE, int THREADS, int PF = 2>
cudaError_t launch_direct(const TrainerDev& a, int grid, cudaStream_t stream) {
  static_assert(kBlockFeatures * 4 == 128, "a bin row of the CTA histogram is 128 bytes");
  const size_t smem = HistSmem<MODE>::kBytes + kFlushBytes + (sizeof(ItemDesc) + 15) / 16 * 16;
  static std::atomic<unsigned long long> configured{0};  // one bit per device
  const cudaError_t err = opt_in_dynamic_smem(configured, hist_build_direct_kernel<MODE, THREADS, PF>, smem);
  if (err != cudaSuccess) return err;
  hist_build_direct_kernel<MODE, THREADS, PF><<<grid, THREADS, smem, stream>>>(a);
  return cudaGetLastError();
}

// Register-direct launch for a mode: 768 threads (bins two groups ahead), 640 (three
// ahead: the deeper ring needs more registers than 768 threads leave) or 512 (two ahead).
template <int MODE>
cudaError_t launch_direct_shape(const TrainerDev& a, int threads, int grid, cudaStream_t stream) {
  if (threads == 512) return launch_direct<MODE, 512>(a, grid, stream);
  if (threads == 640) return launch_direct<MODE, 640, 3>(a, grid, stream);
  return launch_direct<MODE, 768>(a, grid, stream);
}

template <int MODE, int THREADS, int NSTAGE, bool TMA = false>
cudaError_t launch_variant(const TrainerDev& a, int grid, cudaStream_t stream,
                           const CUtensorMap* tmap = nullptr) {
  static_assert(HistSmem<MODE>::kBytes % 128 == 0, "stage slots must stay 128-byte aligned");
  const size_t smem = hist_smem_bytes<MODE, THREADS, NSTAGE, TMA>();
  static std::atomic<unsigned long long> configured{0};  // per variant, one bit per device
  const cudaError_t err = opt_in_dynamic_smem(configured, hist_build_kernel<MODE, THREADS, NSTAGE, TMA>, smem);
  if (err != cudaSuccess) return err;
  static const CUtensorMap kNoMap{};
  hist_build_kernel<MODE, THREADS, NSTAGE, TMA><<<grid, THREADS, smem, stream>>>(a, tmap ? *tmap : kNoMap);
  return cudaGetLastError();
}

}  // namespace

namespace {

// ---- Wide datasets (more than 256 slots per feature) -----------------------------------
//
// The work items of the u8 kernels (build node, row chunk, block of 32 features) over the
// u16 column blocks (a row's block is 64 contiguous bytes). A CTA accumulates `group`
// features of its block at a time (a power of two: as many as the shared-memory budget
// holds) in the u8 kernels' 32-bit limbs per cell ([limb][bin][feature]; exact over the
// item's <= 2^16 rows), then adds the non-empty cells into the node's slot. A warp takes
// 32 gathered rows at a time: lane l quantizes row l's values once, then group / 2 lanes
// per row each load one 4-byte word (two features' bins) of a row, with the row id and the
// limbs shuffled from the quantizing lane, and reduce both features, neighbouring rows in
// opposite order, so that each round's reductions spread over the group's features.
// Features too wide for one feature's cells in shared memory (group 0) add each row
// straight into the slot with 64-bit global atomics.
constexpr uint32_t kWideBatch = 4;  // gathered words in flight per lane
constexpr size_t kWideSmemBytes = 200 * 1024;  // the CTA histogram's limbs
// Fixed-point flushes go through TMA bulk reductions of 8 cells of one feature (192
// bytes), staged by kWideFlushWarps warps in rows after the histogram.
constexpr int kWideFlushWarps = 4;
constexpr size_t kWideStagingBytes = size_t(kWideFlushWarps) * 32 * kFlushRowWords * 8;

template <int MODE>
__host__ __device__ constexpr int wide_words() {  // 32-bit limbs per cell
  return MODE == kModeFixed ? 5 : (MODE == kModeFixedG ? 2 : 3);
}

// Features per shared-memory pass: the largest power of two <= 32 whose cells fit (0: none).
template <int MODE>
uint32_t wide_group(uint32_t slots) {
  const size_t fit = kWideSmemBytes / (size_t(slots) * wide_words<MODE>() * sizeof(uint32_t));
  uint32_t g = kBlockFeatures;
  while (g > fit) g >>= 1;
  return g;
}

__device__ __forceinline__ uint32_t ld_nc_u32(const void* p) {
  uint32_t v;
  asm volatile("ld.global.nc.u32 %0, [%1];\n" : "=r"(v) : "l"(p));
  return v;
}

template <int MODE, int THREADS>
__global__ void __launch_bounds__(THREADS) hist_build_wide_kernel(TrainerDev a, uint32_t group) {
  constexpr int WORDS = wide_words<MODE>();
  constexpr int WARPS = THREADS / 32;
  extern __shared__ __align__(16) uint32_t wsm[];  // [WORDS][slots][group], then the staging rows
  __shared__ uint32_t s_item, s_entry;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const uint32_t n = a.n_rows, nfb = a.nfb, S = a.slots;
  const uint32_t cells = S * group;
  const uint32_t L = group >= 2 ? group / 2 : 1u;  // lanes per row
  const uint32_t R = 32u / L;                      // rows per step
  const uint32_t flip = (uint32_t(lane) / L) & 1u;
  const uint32_t w = uint32_t(lane) % L;           // the lane's word of a row's group
  const uint32_t hist_base = static_cast<uint32_t>(__cvta_generic_to_shared(wsm));
  const uint32_t plane = cells * 4u;               // bytes per limb plane
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
    const float2* gh_seg = a.gh_ordered ? a.gh + seg : nullptr;
    const float2* gh_row = a.gh_ordered ? nullptr : a.gh + size_t(e.tree) * n;
    const uint16_t* bins = a.bins16 + size_t(fb) * n * kBlockFeatures;
    const int kg = a.trees[e.tree].kg;
    const int kh = a.trees[e.tree].kh;
    const long long q_unit_h = MODE == kModeFixedCG ? quantize_f32(1.0f, kh) : 0ll;
    const uint32_t width = min(uint32_t(kBlockFeatures), a.features - fb * kBlockFeatures);
    unsigned long long* dst_base = a.hist + (size_t(e.slot) * a.features + size_t(fb) * kBlockFeatures) * S * 3;
    const uint32_t ntiles = (row_count + 31u) / 32u;
    const uint32_t step = group ? group : width;
    for (uint32_t f0 = 0; f0 < width; f0 += step) {
      const uint32_t gw = min(step, width - f0);
      if (group) {
        uint4* z = reinterpret_cast<uint4*>(wsm);
        for (uint32_t i = tid; i < uint32_t(WORDS) * cells / 4u; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();
      }
      // Row id and values of the lane's row of tile t (zeros past the item's end).
      auto load_row = [&](uint32_t t, uint32_t& r, float2& p) {
        const uint32_t pos = t * 32u + uint32_t(lane);
        r = 0u;
        p = make_float2(0.f, 0.f);
        if (t < ntiles && pos < row_count) {
          r = __ldg(rows + pos);
          r = r < n ? r : 0u;  // row ids are < n by construction
          p = gh_seg ? __ldg(gh_seg + pos) : __ldg(gh_row + r);
        }
      };
      uint32_t r_nxt;
      float2 p_nxt;
      load_row(uint32_t(warp), r_nxt, p_nxt);
      for (uint32_t t = warp; t < ntiles; t += WARPS) {
        const uint32_t pos = t * 32u + uint32_t(lane);
        const uint32_t r = r_nxt;
        const float2 p = p_nxt;
        load_row(t + WARPS, r_nxt, p_nxt);  // the warp's next tile, in flight meanwhile
        if (!group) {  // straight into the slot, each lane its own row
          if (pos < row_count) {
            const long long qg = MODE == kModeFloat ? 0ll : quantize_f32(p.x, kg);
            const long long qh = MODE == kModeFixed ? quantize_f32(p.y, kh) : q_unit_h;
            for (uint32_t j = f0; j < f0 + gw; ++j) {
              const uint32_t b = __ldg(bins + size_t(r) * kBlockFeatures + j);
              if (b >= S) continue;  // the pack checked every bin against its feature's count
              unsigned long long* c = dst_base + (size_t(j) * S + b) * 3;
              if constexpr (MODE == kModeFloat) {
                atomicAdd(c, 1ull);
                atomicAdd(reinterpret_cast<double*>(c + 1), double(p.x));
                atomicAdd(reinterpret_cast<double*>(c + 2), double(p.y));
              } else {
                if constexpr (MODE != kModeFixedG) atomicAdd(c, 1ull);
                atomicAdd(c + 1, (unsigned long long)qg);
                if constexpr (MODE != kModeFixedG) atomicAdd(c + 2, (unsigned long long)qh);
              }
            }
          }
          continue;
        }
        // The row's limbs, as the u8 kernels stage them.
        uint2 v = make_uint2(0u, 0u);
        if (pos < row_count) {
          if constexpr (MODE == kModeFixed) {
            const long long qg = quantize_f32(p.x, kg);
            const long long qh = quantize_f32(p.y, kh);
            const uint32_t glo = uint32_t(qg) & 0xFFFFu, ghi = uint32_t(qg >> 16) & 0xFFFFu;
            const uint32_t hlo = uint32_t(qh) & 0xFFFFu, hhi = uint32_t(qh >> 16) & 0xFFFFu;
            v = make_uint2(glo | (hlo << 16), ghi | (hhi << 16));
          } else if constexpr (MODE == kModeFloat) {
            v = make_uint2(__float_as_uint(p.x), __float_as_uint(p.y));
          } else {
            v = make_uint2(uint32_t(quantize_f32(p.x, kg)), 0u);
          }
        }
        auto accumulate = [&](uint32_t cell, uint32_t vx, uint32_t vy) {
          const uint32_t addr = hist_base + cell * 4u;
          if constexpr (MODE == kModeFixed) {
            red_shared_u32(addr, 1u);
            red_shared_u32(addr + plane, vx & 0xFFFFu);
            red_shared_u32(addr + 2u * plane, uint32_t(int32_t(int16_t(vy & 0xFFFFu))));
            red_shared_u32(addr + 3u * plane, vx >> 16);
            red_shared_u32(addr + 4u * plane, vy >> 16);
          } else if constexpr (MODE == kModeFixedG) {
            red_shared_u32(addr, vx & 0xFFFFu);
            red_shared_u32(addr + plane, uint32_t(int32_t(vx) >> 16));
          } else if constexpr (MODE == kModeFixedCG) {
            red_shared_u32(addr, 1u);
            red_shared_u32(addr + plane, vx & 0xFFFFu);
            red_shared_u32(addr + 2u * plane, uint32_t(int32_t(vx) >> 16));
          } else {
            red_shared_u32(addr, 1u);
            red_shared_f32(addr + plane, __uint_as_float(vx));
            red_shared_f32(addr + 2u * plane, __uint_as_float(vy));
          }
        };
        // Steps in batches of kWideBatch: the batch's gathers are issued together, then
        // reduced. A step's word is that of row st * R + lane / L of the tile.
        for (uint32_t st0 = 0; st0 < L; st0 += kWideBatch) {
          uint32_t word[kWideBatch], bx[kWideBatch], by[kWideBatch];
          bool ok[kWideBatch];
#pragma unroll
          for (uint32_t k = 0; k < kWideBatch; ++k) {
            const uint32_t src = (st0 + k) * R + uint32_t(lane) / L;  // < 32 while st0 + k < L
            const uint32_t src_lane = src & 31u;
            const uint32_t rr = __shfl_sync(0xffffffffu, r, int(src_lane));
            bx[k] = __shfl_sync(0xffffffffu, v.x, int(src_lane));
            by[k] = __shfl_sync(0xffffffffu, v.y, int(src_lane));
            ok[k] = st0 + k < L && t * 32u + src < row_count && 2u * w < gw;
            word[k] = 0u;
            if (ok[k])
              word[k] = group >= 2 ? ld_nc_u32(bins + size_t(rr) * kBlockFeatures + f0 + 2u * w)
                                   : uint32_t(__ldg(bins + size_t(rr) * kBlockFeatures + f0));
          }
#pragma unroll
          for (uint32_t k = 0; k < kWideBatch; ++k) {
            if (!ok[k]) continue;
#pragma unroll
            for (uint32_t i = 0; i < 2; ++i) {
              const uint32_t sel = (i + flip) & 1u;
              const uint32_t fl = 2u * w + sel;
              const uint32_t b = sel ? word[k] >> 16 : word[k] & 0xFFFFu;
              if (fl < gw && b < S) accumulate(b * group + fl, bx[k], by[k]);
            }
          }
        }
      }
      if (group) {
        __syncthreads();
        if constexpr (MODE == kModeFloat) {
          for (uint32_t idx = tid; idx < cells; idx += THREADS) {
            const uint32_t fl = idx % group, b = idx / group;
            if (fl >= gw || wsm[idx] == 0) continue;
            unsigned long long* dst = dst_base + (size_t(f0 + fl) * S + b) * 3;
            atomicAdd(dst + 0, (unsigned long long)wsm[idx]);
            atomicAdd(reinterpret_cast<double*>(dst + 1), double(__uint_as_float(wsm[cells + idx])));
            atomicAdd(reinterpret_cast<double*>(dst + 2), double(__uint_as_float(wsm[2 * cells + idx])));
          }
        } else if (warp < kWideFlushWarps) {
          // Lane (bin group bg, feature fl) of a warp's tile converts 8 consecutive bins of
          // its feature into the slot's 24 words and hands them to one bulk reduction.
          unsigned long long* row = reinterpret_cast<unsigned long long*>(
              reinterpret_cast<unsigned char*>(wsm) + size_t(WORDS) * cells * 4) + (size_t(warp) * 32 + lane) * kFlushRowWords;
          const uint32_t row_addr = static_cast<uint32_t>(__cvta_generic_to_shared(row));
          const uint32_t per_tile = 32u / group;  // bin groups per tile (group divides 32)
          const uint32_t fl = uint32_t(lane) % group, bg = uint32_t(lane) / group;
          for (uint32_t g0 = uint32_t(warp) * per_tile; g0 < S / kFlushBins; g0 += kWideFlushWarps * per_tile) {
            const uint32_t b0 = (g0 + bg) * kFlushBins;  // S / 8 is a multiple of 32
            bulk_wait_read();  // the row's previous bulk reduction has read it
            unsigned long long any = 0;
#pragma unroll
            for (uint32_t j = 0; j < kFlushBins; ++j) {
              const uint32_t idx = (b0 + j) * group + fl;
              unsigned long long c, g, h;
              if constexpr (MODE == kModeFixed) {
                c = wsm[idx];
                g = (unsigned long long)((long long)int32_t(wsm[2 * cells + idx]) * 65536 + (long long)wsm[cells + idx]);
                h = (unsigned long long)((long long)wsm[4 * cells + idx] * 65536 + (long long)wsm[3 * cells + idx]);
              } else if constexpr (MODE == kModeFixedG) {
                c = 0;  // the gradient-only root's count and hessian words are restored afterwards
                g = (unsigned long long)((long long)int32_t(wsm[cells + idx]) * 65536 + (long long)wsm[idx]);
                h = 0;
              } else {
                c = wsm[idx];
                g = (unsigned long long)((long long)int32_t(wsm[2 * cells + idx]) * 65536 + (long long)wsm[cells + idx]);
                h = (unsigned long long)((long long)c * q_unit_h);
              }
              row[3 * j + 0] = c;
              row[3 * j + 1] = g;
              row[3 * j + 2] = h;
              any |= c | g | h;
            }
            if (fl < gw && any != 0ull) {
              asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the row's stores before the bulk read
              bulk_reduce_add_u64(dst_base + (size_t(f0 + fl) * S + b0) * 3, row_addr, kFlushBins * 3 * 8);
              bulk_commit();
            }
          }
          bulk_wait_read();  // the staging rows are free again
        }
        __syncthreads();
      }
    }
    if (tid == 0) {
      atomicAdd(&a.ctl->cells, (unsigned long long)row_count * width);
      if (fb == 0) atomicAdd(&a.ctl->rows_built, (unsigned long long)row_count);
    }
    __syncthreads();
  }
  bulk_wait_all();  // this thread's bulk reductions have reached the slots
}

template <int MODE, int THREADS>
cudaError_t launch_wide(const TrainerDev& a, int grid, cudaStream_t stream) {
  static std::atomic<unsigned long long> configured{0};  // one bit per device
  const cudaError_t err = opt_in_dynamic_smem(configured, hist_build_wide_kernel<MODE, THREADS>,
                                              kWideSmemBytes + kWideStagingBytes);
  if (err != cudaSuccess) return err;
  const uint32_t group = wide_group<MODE>(a.slots);
  const size_t smem = group ? size_t(group) * a.slots * wide_words<MODE>() * sizeof(uint32_t) + kWideStagingBytes : 0;
  hist_build_wide_kernel<MODE, THREADS><<<grid, THREADS, smem, stream>>>(a, group);
  return cudaGetLastError();
}

// Wide launches: 1024 threads, or 512.
template <int MODE>
cudaError_t launch_wide_shape(const TrainerDev& a, int threads, int grid, cudaStream_t stream) {
  if (threads == 512) return launch_wide<MODE, 512>(a, grid, stream);
  return launch_wide<MODE, 1024>(a, grid, stream);
}

}  // namespace

cudaError_t launch_hist_build(const TrainerDev& a, const HistConfig& cfg, int grid,
                              cudaStream_t stream) {
  if (a.slots != uint32_t(kSlots)) {
    if (!a.bins16 || a.slots < uint32_t(kSlots) || a.slots > 65536u) return cudaErrorInvalidValue;
    const int t = cfg.wide_threads;
    if (a.mode == kModeFixedG) return launch_wide_shape<kModeFixedG>(a, t, grid, stream);
    if (a.mode == kModeFixedCG) return launch_wide_shape<kModeFixedCG>(a, t, grid, stream);
    if (a.mode == kModeFixed) return launch_wide_shape<kModeFixed>(a, t, grid, stream);
    return launch_wide_shape<kModeFloat>(a, t, grid, stream);
  }
  const bool row_major_tma = cfg.bins_tmap && a.mode == kModeFixed && a.bins_block_stride == kBlockFeatures &&
                             a.bins_row_stride == uint64_t(a.nfb) * kBlockFeatures;
  if (cfg.direct && a.mode != kModeFloat && !row_major_tma) {
    const int t = a.mode == kModeFixedG ? cfg.root_threads : cfg.threads;
    if (a.mode == kModeFixedG) return launch_direct_shape<kModeFixedG>(a, t, grid, stream);
    if (a.mode == kModeFixedCG) return launch_direct_shape<kModeFixedCG>(a, t, grid, stream);
    return launch_direct_shape<kModeFixed>(a, t, grid, stream);
  }
  // Shared memory: 160 KB (fixed) / 64 KB (gradient only) / 96 KB (float) histogram +
  // stages x threads x 40 B.
  if (a.mode == kModeFixedG) {
    if (cfg.root_threads == 1024) return launch_variant<kModeFixedG, 1024, 2>(a, grid, stream);
    return launch_variant<kModeFixedG, 768, 2>(a, grid, stream);
  }
  if (a.mode == kModeFixedCG) {  // 96 KB histogram: room for 1024 threads
    if (cfg.root_threads == 1024) return launch_variant<kModeFixedCG, 1024, 2>(a, grid, stream);
    return launch_variant<kModeFixedCG, 768, 2>(a, grid, stream);
  }
  if (a.mode == kModeFixed) {
    // Row-major view of the matrix the tensor map describes: gather with TMA.
    const bool tma = cfg.bins_tmap && a.bins_block_stride == kBlockFeatures &&
                     a.bins_row_stride == uint64_t(a.nfb) * kBlockFeatures;
    if (tma && cfg.threads == 768) return launch_variant<kModeFixed, 768, 2, true>(a, grid, stream, cfg.bins_tmap);
    if (tma && cfg.threads == 512 && cfg.stages == 3)
      return launch_variant<kModeFixed, 512, 3, true>(a, grid, stream, cfg.bins_tmap);
    if (tma && cfg.threads == 512) return launch_variant<kModeFixed, 512, 2, true>(a, grid, stream, cfg.bins_tmap);
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

namespace mpsb {

bool encode_bins_tmap(CUtensorMap* map, const uint8_t* bins, uint64_t row_stride, uint32_t n_rows) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                              CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                              CUtensorMapFloatOOBfill);
  static Encode encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return Encode(nullptr);
    return reinterpret_cast<Encode>(fn);
  }();
  if (!encode || !bins || n_rows == 0 || row_stride % 16 != 0) return false;
  // Dimension 0: the row's bytes (feature blocks of 32 bins), dimension 1: rows. A box is
  // one 32-byte feature block of one row (gather4 takes four rows of it).
  const cuuint64_t dims[2] = {row_stride, n_rows};
  const cuuint64_t strides[1] = {row_stride};
  const cuuint32_t box[2] = {uint32_t(kBlockFeatures), 1u};
  const cuuint32_t elem[2] = {1u, 1u};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t*>(bins), dims, strides, box,
                elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace mpsb
