// Shared definitions for the sm_103a kernels of the ExSHalos mock path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/exh_gb300.h"

#define EXH_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) {                                 \
      exh_set_error_msg(cudaGetErrorString(_e), __FILE__, __LINE__); \
      return EXH_E_CUDA;                                     \
    }                                                        \
  } while (0)

#define EXH_TRY(expr)                 \
  do {                                \
    int _s = (expr);                  \
    if (_s != EXH_OK) return _s;      \
  } while (0)

// last error text, per host thread
void exh_set_error_msg(const char* msg, const char* file, int line);

// periodic neighbour index, the cysum of exshalos_h.c:21-32
__host__ __device__ __forceinline__ int exh_wrap(int i, int j, int nd) {
  int r = i + j;
  if (r >= nd) r -= nd;
  if (r < 0) r += nd;
  return r;
}

// (i, j, k) of the row-major cell index of an n0 x n1 x n2 grid of ng cells;
// 32-bit divisions while the index fits
__device__ __forceinline__ void cell_ijk(size_t cell, size_t ng, int n1, int n2, int* i, int* j, int* k) {
  if (ng <= 0xffffffffull) {
    const unsigned c32 = (unsigned)cell, r = c32 / (unsigned)n2;
    *k = (int)(c32 - r * (unsigned)n2);
    *j = (int)(r % (unsigned)n1);
    *i = (int)(r / (unsigned)n1);
  } else {
    *k = (int)(cell % n2);
    const size_t r = cell / n2;
    *j = (int)(r % n1);
    *i = (int)(r / n1);
  }
}

__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

static inline unsigned exh_div_up(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

constexpr int EXH_NUM_SMS = 152;   // GB300: 2 dies x 76 SMs
