// FP32 restatements of sums the reference forms in double, for kernels that
// would otherwise spend FP64 operations (a small fraction of the FP32 rate
// on this GPU) on every term.  Every operation is an explicitly rounded IEEE
// float operation, so the host build (plain C++, compiled without FMA
// contraction) gives the same bits and a host program can check the
// error bounds against FP64.
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define EXH_F32_HD __host__ __device__ __forceinline__
#else
#define EXH_F32_HD inline
#endif

namespace exh {

EXH_F32_HD float f32_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
EXH_F32_HD float f32_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
EXH_F32_HD float f32_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
EXH_F32_HD float f32_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

// Compensated (Neumaier) float sum, kept as s + c: its error is about 2^-24
// of the total plus 2^-48 of the sum of magnitudes.  value() = s + c exactly
// in double.
struct FSum {
  float s = 0.f, c = 0.f;
  EXH_F32_HD void add(float x) {
    const float t = f32_add(s, x);
    c = f32_add(c, std::fabs(s) >= std::fabs(x) ? f32_add(f32_sub(s, t), x) : f32_add(f32_sub(x, t), s));
    s = t;
  }
  EXH_F32_HD double value() const { return (double)s + (double)c; }
};

// diag - x^2 - y^2 - z^2, which the reference forms in double from float
// operands (pow(., 2.0), lpt.c:134).  Each square is split exactly into
// hi + lo by an FMA, the running value is kept as s + c with s updated by an
// error-free TwoSum (Knuth), and the sum is rounded once at the end: the
// error before that rounding is about 2^-47 of the largest term.
EXH_F32_HD float source_combine(float diag, float x, float y, float z) {
  float s = diag, c = 0.f;
  const float p[3] = {x, y, z};
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int a = 0; a < 3; a++) {
    const float hi = f32_mul(p[a], p[a]);
    const float lo = f32_fma(p[a], p[a], -hi);            // p^2 = hi + lo exactly
    const float t = f32_sub(s, hi);
    const float bb = f32_sub(t, s);                        // TwoSum of s and -hi
    const float e = f32_add(f32_sub(s, f32_sub(t, bb)), f32_sub(-hi, bb));
    s = t;
    c = f32_sub(f32_add(c, e), lo);
  }
  return f32_add(s, c);
}

}  // namespace exh
