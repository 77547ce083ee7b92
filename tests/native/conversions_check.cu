// Checks the software IEEE conversions of device.cuh (s64_to_f32_rn, f64_to_f32_rn,
// f64_finite on 2^26 seeded inputs per family) bit for bit against the hardware
// conversions, plus the edge cases: ties at every rounding
// position, the float overflow threshold, the subnormal range and its boundaries, signed
// zeros, infinities and NaNs.
// Exit status 0 when every result matches; prints the first mismatch otherwise.
#include <cstdio>
#include <cstdint>

#include "device.cuh"

using namespace mpsb;

struct Report {
  unsigned long long mismatches;
  unsigned long long first_input;
  uint32_t first_got, first_want, first_family;
};

__device__ __forceinline__ unsigned long long mix(unsigned long long z) {  // splitmix64
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ void record(Report* r, uint32_t family, unsigned long long in, uint32_t got,
                       uint32_t want) {
  if (atomicAdd(&r->mismatches, 1ull) == 0) {
    r->first_input = in;
    r->first_got = got;
    r->first_want = want;
    r->first_family = family;
  }
}

// family 0..2: int64 inputs; 3..6: double inputs.
__device__ unsigned long long make_input(uint32_t family, unsigned long long i) {
  const unsigned long long h = mix(i * 7 + family);
  const unsigned long long h2 = mix(h);
  switch (family) {
    case 0:  // uniformly random bit patterns
      return h;
    case 1: {  // random magnitude with a random leading-bit position
      const int top = int(h2 % 64);
      unsigned long long v = top == 63 ? h : (h & ((2ull << top) - 1ull)) | (1ull << top);
      return (h2 >> 7) & 1 ? (unsigned long long)(0 - (long long)v) : v;
    }
    case 2: {  // exact ties and their neighbours at a random rounding position
      const int top = 24 + int(h2 % 39);  // leading bit 24..62
      const int s = top - 23;
      unsigned long long v = (1ull << top) | (h & ((1ull << top) - 1ull));
      v &= ~((1ull << s) - 1ull);
      v |= 1ull << (s - 1);  // exactly half an ulp
      v += (unsigned long long)(int(h2 >> 8) % 3) - 1ull;  // -1, 0, +1
      return (h2 >> 11) & 1 ? (unsigned long long)(0 - (long long)v) : v;
    }
    case 3:  // random double bit patterns
      return h;
    case 4: {  // exponents around the float range, random mantissa and sign
      const unsigned long long e = 1023 - 160 + (h2 % 300);
      return (h & 0x800FFFFFFFFFFFFFull) | (e << 52);
    }
    case 5: {  // ties at the float rounding position (normal and subnormal results)
      const unsigned long long e = 1023 - 152 + (h2 % 285);
      unsigned long long m = h & 0xFFFFFFFFFFFFFull;
      const int E = int(e) - 1023;
      const int s = E >= -126 ? 29 : -E - 97;  // bits below the float ulp
      if (s <= 52) {
        m &= ~((1ull << s) - 1ull);
        m |= 1ull << (s - 1);
        m += (unsigned long long)(int(h2 >> 9) % 3) - 1ull;
        m &= 0xFFFFFFFFFFFFFull;
      }
      return (h & 0x8000000000000000ull) | (e << 52) | m;
    }
    default: {  // small edge list, repeated
      const unsigned long long edges[] = {
          0x0000000000000000ull, 0x8000000000000000ull, 0x7FF0000000000000ull,
          0xFFF0000000000000ull, 0x7FF8000000000000ull, 0x7FF0000000000001ull,
          0x47EFFFFFE0000000ull,  // FLT_MAX
          0x47EFFFFFF0000000ull,  // FLT_MAX + half an ulp: ties to infinity
          0x47EFFFFFEFFFFFFFull,  // just below that tie: FLT_MAX
          0x47EFFFFFE0000001ull, 0x3810000000000000ull,  // 2^-126
          0x380FFFFFF0000000ull,  // 2^-126 - 2^-151
          0x36A0000000000000ull,  // 2^-149
          0x3690000000000000ull,  // 2^-150: tie to zero
          0x3690000000000001ull,  // just above: rounds to 2^-149
          0x3680000000000000ull,  // 2^-151
          0x0000000000000001ull, 0x000FFFFFFFFFFFFFull, 0x0010000000000000ull,
          0x3FF0000010000000ull, 0x3FF0000030000000ull, 0xBFF0000010000000ull};
      return edges[i % (sizeof(edges) / sizeof(edges[0]))];
    }
  }
}

__global__ void check_kernel(uint32_t family, unsigned long long n, Report* r) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long in = make_input(family, i);
    if (family <= 2) {
      const long long q = (long long)in;
      const uint32_t got = __float_as_uint(s64_to_f32_rn(q));
      const uint32_t want = __float_as_uint(__ll2float_rn(q));
      if (got != want) record(r, family, in, got, want);
    } else {
      const double x = __longlong_as_double((long long)in);
      const float gf = f64_to_f32_rn(x), wf = __double2float_rn(x);
      const uint32_t got = __float_as_uint(gf), want = __float_as_uint(wf);
      const bool same = got == want || (isnan(gf) && isnan(wf));
      if (!same) record(r, family, in, got, want);
      if (f64_finite(x) != bool(isfinite(x))) record(r, 100 + family, in, f64_finite(x), isfinite(x));
    }
  }
}

int main() {
  Report* r = nullptr;
  if (cudaMalloc(&r, sizeof(Report)) != cudaSuccess) return 2;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  int failures = 0;
  for (uint32_t family = 0; family <= 6; ++family) {
    cudaMemset(r, 0, sizeof(Report));
    const unsigned long long n = family == 6 ? 4096 : (1ull << 26);
    check_kernel<<<sms * 8, 256>>>(family, n, r);
    Report h{};
    if (cudaMemcpy(&h, r, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
    std::printf("family %u: %llu inputs, %llu mismatches\n", family, n, h.mismatches);
    if (h.mismatches) {
      std::printf("  first: family %u input 0x%016llx got 0x%08x want 0x%08x\n", h.first_family,
                  h.first_input, h.first_got, h.first_want);
      ++failures;
    }
  }
  cudaFree(r);
  return failures ? 1 : 0;
}
