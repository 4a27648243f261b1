// Division of 32-bit unsigned integers by a divisor fixed at launch, as a
// multiply-high and two shifts (Granlund and Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994, the round-up method
// for N = 32): with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1,
//   t = mulhi(m, x),  x / d = (t + ((x - t) >> min(l, 1))) >> max(l - 1, 0)
// for every 32-bit x and every d >= 1.  Plain C++ as well, so that a host
// program can check it against the hardware division.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define EXH_ID_HD __host__ __device__ __forceinline__
#else
#define EXH_ID_HD inline
#endif

namespace exh {

struct FastDiv {
  uint32_t d = 1, m = 1;
  int s1 = 0, s2 = 0;
};

inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  int l = 0;
  while ((1ull << l) < d) l++;
  f.d = d;
  f.m = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / d) + 1ull);
  f.s1 = l < 1 ? l : 1;
  f.s2 = l > 1 ? l - 1 : 0;
  return f;
}

EXH_ID_HD uint32_t fd_div(uint32_t x, const FastDiv& f) {
#ifdef __CUDA_ARCH__
  const uint32_t t = __umulhi(x, f.m);
#else
  const uint32_t t = (uint32_t)(((uint64_t)x * f.m) >> 32);
#endif
  return (t + ((x - t) >> f.s1)) >> f.s2;
}

}  // namespace exh
