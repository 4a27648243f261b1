// Device-wide exclusive prefix sum of 32-bit counts (three passes:
// per-block sums, one-block scan of the sums, per-block rescan).
#pragma once
#include "exh_common.cuh"

namespace exh {

constexpr int SCAN_T = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_T * SCAN_ITEMS;

// block-wide exclusive scan of one value per thread; returns the block total
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* warp_sums, T& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    T s = lane < nw ? warp_sums[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) warp_sums[lane] = s;
  }
  __syncthreads();
  total = warp_sums[nw - 1];
  const T before = w > 0 ? warp_sums[w - 1] : T(0);
  __syncthreads();
  return before + x - v;
}

template <typename T>
__global__ void k_scan_tile_sums(const T* __restrict__ in, size_t n, T* __restrict__ sums) {
  __shared__ T ws[32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  T s = 0;
  for (int i = 0; i < SCAN_ITEMS; i++) {
    const size_t idx = base + (size_t)i * SCAN_T + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  T tot;
  block_exclusive_scan<T>(s, ws, tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void k_scan_sums(T* __restrict__ sums, int nb, T* __restrict__ total) {
  __shared__ T ws[32];
  __shared__ T carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += blockDim.x) {
    const int i = base + threadIdx.x;
    T v = i < nb ? sums[i] : T(0);
    T tot;
    T ex = block_exclusive_scan<T>(v, ws, tot);
    if (i < nb) sums[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

template <typename T>
__global__ void k_scan_apply(const T* __restrict__ in, size_t n, const T* __restrict__ sums, T* __restrict__ out) {
  __shared__ T ws[32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  T v[SCAN_ITEMS];
  T s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    const size_t idx = base + i;
    v[i] = idx < n ? in[idx] : T(0);
    s += v[i];
  }
  T tot;
  T run = block_exclusive_scan<T>(s, ws, tot) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    const size_t idx = base + i;
    if (idx < n) out[idx] = run;
    run += v[i];
  }
}

void count_launch(int n);

// out[i] = sum_{j<i} in[j]; *total_dev = sum of all.  scratch: >= n/SCAN_TILE+1
template <typename T>
inline cudaError_t exclusive_scan(const T* in, T* out, size_t n, T* scratch, T* total_dev, cudaStream_t st) {
  const unsigned nb = (unsigned)((n + SCAN_TILE - 1) / SCAN_TILE);
  if (nb == 0) {
    if (total_dev) return cudaMemsetAsync(total_dev, 0, sizeof(T), st);
    return cudaSuccess;
  }
  k_scan_tile_sums<T><<<nb, SCAN_T, 0, st>>>(in, n, scratch);
  k_scan_sums<T><<<1, 1024, 0, st>>>(scratch, (int)nb, total_dev);
  k_scan_apply<T><<<nb, SCAN_T, 0, st>>>(in, n, scratch, out);
  count_launch(3);
  return cudaGetLastError();
}

}  // namespace exh
