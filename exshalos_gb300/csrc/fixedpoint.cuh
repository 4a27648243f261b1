// Conversions between float weights and the 64-bit fixed-point quanta of the
// CIC accumulator (2^-40), in 32/64-bit integer arithmetic.  They give the
// bits of the FP64 expressions
//   quanta: __double2ull_rn((double)w * 2^40)        (w >= 0, finite)
//   value:  (float)((double)q * 2^-40)               (q: u64 sum)
// without the FP64 pipe, which runs at a small fraction of the integer and
// FP32 rates on this GPU.  Plain C++ as well, so that a host program can
// check them against the FP64 expressions.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define EXH_FP_HD __host__ __device__ __forceinline__
#else
#define EXH_FP_HD inline
#endif

namespace exh {

EXH_FP_HD uint32_t fp_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}

EXH_FP_HD float fp_from_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

EXH_FP_HD int fp_bitlen64(uint64_t v) {   // v > 0
#ifdef __CUDA_ARCH__
  return 64 - __clzll((long long)v);
#else
  return 64 - __builtin_clzll(v);
#endif
}

// v / 2^r rounded to nearest, ties to even (0 < r < 64)
EXH_FP_HD uint64_t fp_shr_rne(uint64_t v, int r) {
  const uint64_t q = v >> r, rem = v & ((1ull << r) - 1ull), half = 1ull << (r - 1);
  return q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
}

// round(w 2^40), ties to even, for a finite w >= 0 (0 for a negative w)
EXH_FP_HD uint64_t fp_quanta40(float w) {
  const uint32_t u = fp_bits(w);
  if (u >> 31) return 0ull;
  const int E = (int)(u >> 23);
  if (E == 0) return 0ull;                          // zero or subnormal: below 2^-126
  const uint64_t M = (u & 0x7fffffu) | 0x800000u;   // w = M 2^(E - 150)
  const int s = E - 110;                            // w 2^40 = M 2^s
  if (s >= 0) return M << s;
  if (-s > 24) return 0ull;                         // M 2^s < 1/2
  return fp_shr_rne(M, -s);
}

// (float)((double)q 2^-40): q rounded to 53 bits, then to 24, ties to even
// at both steps, as the two conversions do
EXH_FP_HD float fp_value40(uint64_t q) {
  if (q == 0ull) return 0.f;
  int e = -40;
  int n = fp_bitlen64(q);
  if (n > 53) {
    q = fp_shr_rne(q, n - 53);
    e += n - 53;
    n = fp_bitlen64(q);                             // 53, or 54 after a carry (q = 2^53)
  }
  if (n > 24) {
    q = fp_shr_rne(q, n - 24);
    e += n - 24;
  }
  // q <= 2^24 is exact in float; 2^e (-40 <= e <= 23) is a normal float
  return (float)(uint32_t)q * fp_from_bits((uint32_t)(e + 127) << 23);
}

}  // namespace exh
