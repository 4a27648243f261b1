// Four-step FFT passes held in registers.
//
// A length n = N1 * N2 transform of each column of a tile runs as
//   step 1: N2 threads per column, each an N1-point DFT in registers over the
//           elements j2 + N2 j1, times the twiddle W_n^(j2 k1);
//   one shared-memory transpose;
//   step 3: N1 threads per column, each an N2-point DFT in registers,
//           output index k1 + N1 k2.
// Compared with a shared-memory Stockham network this touches shared memory
// once, needs one buffer (32 KB for 16 columns of 256) and keeps 16 loads in
// flight per thread.  Register DFTs are composite Cooley-Tukey on radices
// 2, 3, 4 and 8; their twiddles come from the axis table W_n^m.
#pragma once
#include "fft.cuh"

namespace exh {

template <int N>
struct RDft {
  static constexpr int A = (N % 4 == 0) ? 4 : ((N % 3 == 0) ? 3 : 2);
  static constexpr int B = N / A;
  // w(m) = (cos, sin) of 2 pi m / N for 0 <= m < N
  template <class TW>
  __device__ __forceinline__ static void run(float2* v, float sgn, TW w) {
    float2 t[N];
#pragma unroll
    for (int j2 = 0; j2 < B; j2++) {
      float2 a[A];
#pragma unroll
      for (int j1 = 0; j1 < A; j1++) a[j1] = v[j2 + B * j1];
      dft<A>(a, sgn);
#pragma unroll
      for (int k1 = 0; k1 < A; k1++) {
        float2 x = a[k1];
        if (j2 * k1 != 0) {
          const float2 c = w(j2 * k1);
          x = cmul(x, make_float2(c.x, sgn * c.y));
        }
        t[k1 * B + j2] = x;
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < A; k1++) {
      float2 b[B];
#pragma unroll
      for (int j2 = 0; j2 < B; j2++) b[j2] = t[k1 * B + j2];
      RDft<B>::run(b, sgn, [w](int m) { return w(m * A); });
#pragma unroll
      for (int k2 = 0; k2 < B; k2++) v[k1 + A * k2] = b[k2];
    }
  }
};
template <> struct RDft<2> { template <class TW> __device__ __forceinline__ static void run(float2* v, float s, TW) { dft<2>(v, s); } };
template <> struct RDft<3> { template <class TW> __device__ __forceinline__ static void run(float2* v, float s, TW) { dft<3>(v, s); } };
template <> struct RDft<4> { template <class TW> __device__ __forceinline__ static void run(float2* v, float s, TW) { dft<4>(v, s); } };
template <> struct RDft<8> { template <class TW> __device__ __forceinline__ static void run(float2* v, float s, TW) { dft<8>(v, s); } };

constexpr int FS_THREADS = 256;

template <int N1, int N2>
struct FsShape {
  static constexpr int n = N1 * N2;
  static constexpr int NMAX = N1 > N2 ? N1 : N2;
  static constexpr int W = (FS_THREADS / NMAX) < 16 ? (FS_THREADS / NMAX) : 16;   // columns per tile
  static constexpr int R = FS_THREADS / NMAX;                                     // rows per tile
};

// Strided pass over data [outer][n][inner]: a tile of W columns.  Column q
// of the flattened (outer, inner) index is (q / inner, q % inner), so a tile
// may end one outer row and start the next (two contiguous runs per row):
// with inner = n/2 + 1 every tile is full, where tiles within one outer row
// would leave one column in the last tile of each row.
template <int N1, int N2, class Src, class Dst>
__global__ void __launch_bounds__(FS_THREADS, 4)
k_fft4_strided(Src src, Dst dst, const float2* __restrict__ tw, float sgn, int inner, int ncol) {
  using S = FsShape<N1, N2>;
  constexpr int W = S::W;
  __shared__ float2 sm[S::n * W];
  const int c = threadIdx.x % W, jj = threadIdx.x / W;
  const int q = blockIdx.x * W + c;
  const bool ok = q < ncol;
  const int o = q / inner, i = q - o * inner;
  if (jj < N2) {
    float2 v[N1];
#pragma unroll
    for (int j1 = 0; j1 < N1; j1++) v[j1] = ok ? src(o, jj + N2 * j1, i) : make_float2(0.f, 0.f);
    RDft<N1>::run(v, sgn, [tw](int m) { return __ldg(&tw[m * N2]); });
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) {
      float2 x = v[k1];
      if (k1 != 0 && jj != 0) x = cmul(x, tw_get(tw, jj * k1, sgn));
      sm[(k1 * N2 + jj) * W + c] = x;
    }
  }
  __syncthreads();
  if (jj < N1) {
    float2 u[N2];
#pragma unroll
    for (int j2 = 0; j2 < N2; j2++) u[j2] = sm[(jj * N2 + j2) * W + c];
    RDft<N2>::run(u, sgn, [tw](int m) { return __ldg(&tw[m * N1]); });
    if (ok) {
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) dst(o, jj + N1 * k2, i, u[k2]);
    }
  }
}

// Strided pass of length 512 = 8 x 8 x 8.  The two-factor split 32 x 16
// would hold a 32-point DFT per thread (beyond the register budget at full
// occupancy: it spills) and leave half the threads idle in its first step;
// here 64 threads per column each run three 8-point DFTs:
//   A: j = q + 64 j1 (q < 64): DFT over j1 -> k1, times W_512^(q k1);
//   B: for each k1, q = r + 8 s: DFT over s -> k2a, times W_64^(r k2a);
//   C: for each (k1, k2a): DFT over r -> k2b; output k1 + 8 k2a + 64 k2b,
// with two shared-memory exchanges.  Positions carry one float2 of padding
// per 8, so the four positions a warp touches at once in every exchange
// alternate between the two bank halves.
constexpr int F512_W = 8;                   // columns per tile: 64 B row segments
constexpr int F512_T = 64 * F512_W;
__device__ __forceinline__ int f512_at(int p, int c) { return (p + (p >> 3)) * F512_W + c; }

// The three stages for column c of a tile, thread q < 64 of that column;
// ld(j) returns element j of the column.  On return v[k2b] holds output
// k1 + 8 k2a + 64 k2b with k1 = q >> 3, k2a = q & 7; sm (f512_at layout,
// (512 + 64) F512_W float2) may be written again after a barrier.
// f512_core: the same from v[j1] = element q + 64 j1 already loaded.
__device__ __forceinline__ void f512_core(float2 (&v)[8], float2* sm, const float2* __restrict__ tw, float sgn,
                                          int c, int q) {
  dft<8>(v, sgn);
#pragma unroll
  for (int k1 = 0; k1 < 8; k1++) {
    float2 x = v[k1];
    if (k1 != 0 && q != 0) x = cmul(x, tw_get(tw, q * k1, sgn));
    sm[f512_at(k1 * 64 + q, c)] = x;
  }
  __syncthreads();
  {
    const int k1 = q >> 3, r = q & 7;
#pragma unroll
    for (int s = 0; s < 8; s++) v[s] = sm[f512_at(k1 * 64 + r + 8 * s, c)];
    __syncthreads();
    dft<8>(v, sgn);
#pragma unroll
    for (int k2a = 0; k2a < 8; k2a++) {
      float2 x = v[k2a];
      if (k2a != 0 && r != 0) x = cmul(x, tw_get(tw, 8 * r * k2a, sgn));
      sm[f512_at(k1 * 64 + 8 * k2a + r, c)] = x;
    }
  }
  __syncthreads();
  {
    const int k1 = q >> 3, k2a = q & 7;
#pragma unroll
    for (int r = 0; r < 8; r++) v[r] = sm[f512_at(k1 * 64 + 8 * k2a + r, c)];
    dft<8>(v, sgn);
  }
}

template <class Load>
__device__ __forceinline__ void f512_run(Load ld, float2* sm, const float2* __restrict__ tw, float sgn, int c,
                                         int q, float2 (&v)[8]) {
#pragma unroll
  for (int j1 = 0; j1 < 8; j1++) v[j1] = ld(q + 64 * j1);
  f512_core(v, sm, tw, sgn, c, q);
}

// columns over the flattened (outer, inner) index, as k_fft4_strided
template <class Src, class Dst>
__global__ void __launch_bounds__(F512_T, 3)
k_fft8_strided512(Src src, Dst dst, const float2* __restrict__ tw, float sgn, int inner, int ncol) {
  __shared__ float2 sm[(512 + 64) * F512_W];
  const int c = threadIdx.x % F512_W, q = threadIdx.x / F512_W;
  const int col = blockIdx.x * F512_W + c;
  const bool ok = col < ncol;
  const int o = col / inner, i = col - o * inner;
  float2 v[8];
  f512_run([&](int j) { return ok ? src(o, j, i) : make_float2(0.f, 0.f); }, sm, tw, sgn, c, q, v);
  if (ok) {
    const int k1 = q >> 3, k2a = q & 7;
#pragma unroll
    for (int k2b = 0; k2b < 8; k2b++) dst(o, k1 + 8 * k2a + 64 * k2b, i, v[k2b]);
  }
}

// Row stride (float2) of the row kernels' shared memory: room for the
// padded intermediate of fs_rows_smem, and == 8 (mod 16) so that the 4 or 2
// rows a warp touches at once fall on disjoint bank pairs.
template <int N1, int N2>
struct FsRows {
  static constexpr int M = N1 * N2;
  static constexpr int PAD = (N2 % 2 == 0) ? 1 : 0;   // odd group stride: conflict-free columns
  static constexpr int NEED = (N1 * (N2 + PAD) > M + 1) ? N1 * (N2 + PAD) : M + 1;
  static constexpr int LDA = NEED + ((8 - NEED % 16) + 16) % 16;
};

// Four-step transform of R rows of length M = N1 N2 held in shared memory
// a[b * lda + m]; result in natural order in the same place.  The
// intermediate (after the twiddles) is stored with one float2 of padding
// per group of N2, so the column reads of the second step hit distinct
// banks.
template <int N1, int N2>
__device__ __forceinline__ void fs_rows_smem(float2* a, int lda, const float2* __restrict__ twM, float sgn) {
  using S = FsShape<N1, N2>;
  constexpr int R = S::R;
  constexpr int G = N2 + FsRows<N1, N2>::PAD;
  float2 v[N1];
  {
    const int b = threadIdx.x / N2, jj = threadIdx.x % N2;
    if (b < R) {
#pragma unroll
      for (int j1 = 0; j1 < N1; j1++) v[j1] = a[b * lda + jj + N2 * j1];
      RDft<N1>::run(v, sgn, [twM](int m) { return __ldg(&twM[m * N2]); });
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++)
        if (jj != 0) v[k1] = cmul(v[k1], tw_get(twM, jj * k1, sgn));
    }
    __syncthreads();
    if (b < R) {
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) a[b * lda + k1 * G + jj] = v[k1];
    }
    __syncthreads();
  }
  {
    const int b = threadIdx.x / N1, kk = threadIdx.x % N1;
    float2 u[N2];
    if (b < R) {
#pragma unroll
      for (int j2 = 0; j2 < N2; j2++) u[j2] = a[b * lda + kk * G + j2];
      RDft<N2>::run(u, sgn, [twM](int m) { return __ldg(&twM[m * N1]); });
    }
    __syncthreads();
    if (b < R) {
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) a[b * lda + kk + N1 * k2] = u[k2];
    }
    __syncthreads();
  }
}

// z pass, real -> half complex, four-step on M = N1 N2
template <int N1, int N2, class Src, class Dst>
__global__ void __launch_bounds__(FS_THREADS)
k_fft4_r2c_rows(Src src, Dst dst, const float2* __restrict__ twM, const float2* __restrict__ twN, size_t rows) {
  using S = FsShape<N1, N2>;
  constexpr int M = S::n, R = S::R, LDA = FsRows<N1, N2>::LDA;
  extern __shared__ float2 a[];                    // R * LDA
  const size_t r0 = (size_t)blockIdx.x * R;
  const int nb = (int)min((size_t)R, rows - r0);
#pragma unroll
  for (int t = threadIdx.x; t < R * M; t += FS_THREADS) {
    const int b = t / M, m = t % M;
    a[b * LDA + m] = (b < nb) ? src(r0 + b, m) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  fs_rows_smem<N1, N2>(a, LDA, twM, -1.f);
  const int nc = M + 1;
  for (int t = threadIdx.x; t < R * nc; t += blockDim.x) {
    const int b = t / nc, k = t % nc;
    if (b >= nb) continue;
    const float2 zk = a[b * LDA + (k == M ? 0 : k)];
    const float2 zm = cconj(a[b * LDA + (k == 0 ? 0 : M - k)]);
    const float2 A = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y));
    const float2 d = csub(zk, zm);
    const float2 Bv = make_float2(0.5f * d.y, -0.5f * d.x);
    dst(r0 + b, k, cadd(A, cmul(tw_get(twN, k, -1.f), Bv)));
  }
}

// z pass, half complex -> real, four-step on M = N1 N2
template <int N1, int N2, class Src, class Dst>
__global__ void __launch_bounds__(FS_THREADS)
k_fft4_c2r_rows(Src src, Dst dst, const float2* __restrict__ twM, const float2* __restrict__ twN, size_t rows) {
  using S = FsShape<N1, N2>;
  constexpr int M = S::n, R = S::R, LDA = FsRows<N1, N2>::LDA, nc = M + 1;
  extern __shared__ float2 x[];                    // 2 * R * LDA
  float2* a = x + R * LDA;
  const size_t r0 = (size_t)blockIdx.x * R;
  const int nb = (int)min((size_t)R, rows - r0);
#pragma unroll
  for (int t = threadIdx.x; t < R * nc; t += FS_THREADS) {
    const int b = t / nc, k = t % nc;
    float2 v = (b < nb) ? src(r0 + b, k) : make_float2(0.f, 0.f);
    if (k == 0 || k == M) v.y = 0.f;
    x[b * LDA + k] = v;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < R * M; t += blockDim.x) {
    const int b = t / M, k = t % M;
    const float2 xk = x[b * LDA + k];
    const float2 xm = cconj(x[b * LDA + (M - k)]);
    const float2 d = cmul(tw_get(twN, k, 1.f), csub(xk, xm));
    a[b * LDA + k] = make_float2(xk.x + xm.x - d.y, xk.y + xm.y + d.x);
  }
  __syncthreads();
  fs_rows_smem<N1, N2>(a, LDA, twM, 1.f);
  for (int t = threadIdx.x; t < R * M; t += blockDim.x) {
    const int b = t / M, m = t % M;
    if (b < nb) dst(r0 + b, m, a[b * LDA + m]);
  }
}

// supported four-step splits: returns N1 * 1000 + N2, or 0
inline int fs_split(int n) {
  switch (n) {
    case 16: return 4 * 1000 + 4;
    case 24: return 8 * 1000 + 3;
    case 32: return 8 * 1000 + 4;
    case 48: return 8 * 1000 + 6;
    case 64: return 8 * 1000 + 8;
    case 96: return 8 * 1000 + 12;
    case 128: return 16 * 1000 + 8;
    case 192: return 16 * 1000 + 12;
    case 256: return 16 * 1000 + 16;
    case 512: return 32 * 1000 + 16;
    default: return 0;
  }
}

#define EXH_FS_CASES(X) \
  X(4, 4) X(8, 3) X(8, 4) X(8, 6) X(8, 8) X(8, 12) X(16, 8) X(16, 12) X(16, 16) X(32, 16)
// strided passes: length 512 runs k_fft8_strided512 instead
#define EXH_FS_STRIDED_CASES(X) \
  X(4, 4) X(8, 3) X(8, 4) X(8, 6) X(8, 8) X(8, 12) X(16, 8) X(16, 12) X(16, 16)

template <class Src, class Dst>
inline bool launch_fs_strided(Src src, Dst dst, int n, const float2* tw, float sgn, int outer, int inner,
                              cudaStream_t st, cudaError_t* err) {
  const int ncol = outer * inner;             // at most 512 x 257 x 512 columns
  if (n == 512) {
    k_fft8_strided512<Src, Dst><<<exh_div_up(ncol, F512_W), F512_T, 0, st>>>(src, dst, tw, sgn, inner, ncol);
    *err = cudaGetLastError();
    return true;
  }
  switch (fs_split(n)) {
#define X(a, b)                                                                     \
  case a * 1000 + b: {                                                              \
    k_fft4_strided<a, b, Src, Dst><<<exh_div_up(ncol, FsShape<a, b>::W), FS_THREADS, 0, st>>>(src, dst, tw, sgn, \
                                                                                          inner, ncol); \
    *err = cudaGetLastError();                                                      \
    return true;                                                                    \
  }
    EXH_FS_STRIDED_CASES(X)
#undef X
    default: return false;
  }
}

template <class Src, class Dst>
inline bool launch_fs_r2c(Src src, Dst dst, int M, const float2* twM, const float2* twN, size_t rows,
                          cudaStream_t st, cudaError_t* err) {
  switch (fs_split(M)) {
#define X(a, b)                                                                               \
  case a * 1000 + b: {                                                                        \
    const size_t sm = sizeof(float2) * FsShape<a, b>::R * FsRows<a, b>::LDA;                   \
    *err = set_smem(k_fft4_r2c_rows<a, b, Src, Dst>, sm);                                     \
    if (*err != cudaSuccess) return true;                                                     \
    k_fft4_r2c_rows<a, b, Src, Dst><<<exh_div_up(rows, FsShape<a, b>::R), FS_THREADS, sm, st>>>(src, dst, twM, twN, rows); \
    *err = cudaGetLastError();                                                                \
    return true;                                                                              \
  }
    EXH_FS_CASES(X)
#undef X
    default: return false;
  }
}

template <class Src, class Dst>
inline bool launch_fs_c2r(Src src, Dst dst, int M, const float2* twM, const float2* twN, size_t rows,
                          cudaStream_t st, cudaError_t* err) {
  switch (fs_split(M)) {
#define X(a, b)                                                                               \
  case a * 1000 + b: {                                                                        \
    const size_t sm = 2 * sizeof(float2) * FsShape<a, b>::R * FsRows<a, b>::LDA;              \
    *err = set_smem(k_fft4_c2r_rows<a, b, Src, Dst>, sm);                                     \
    if (*err != cudaSuccess) return true;                                                     \
    k_fft4_c2r_rows<a, b, Src, Dst><<<exh_div_up(rows, FsShape<a, b>::R), FS_THREADS, sm, st>>>(src, dst, twM, twN, rows); \
    *err = cudaGetLastError();                                                                \
    return true;                                                                              \
  }
    EXH_FS_CASES(X)
#undef X
    default: return false;
  }
}

}  // namespace exh

namespace exh {

// Pass launchers: the four-step kernels for the sizes they cover, the
// shared-memory Stockham kernels otherwise.
template <class Src, class Dst>
inline cudaError_t launch_strided(Src src, Dst dst, const RadixPlan& pl, const float2* tw, float sgn, int outer,
                                  int inner, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  {
    KTimer kt(KC_FFT_STRIDED, st, (double)pl.n * inner * outer * (io_bytes<Src>() + io_bytes<Dst>()));
    if (launch_fs_strided(src, dst, pl.n, tw, sgn, outer, inner, st, &e)) {
      count_launch(1);
      return e;
    }
  }
  return launch_strided_sh(src, dst, pl, tw, sgn, outer, inner, st);
}

template <class Src, class Dst>
inline cudaError_t launch_r2c_rows(Src src, Dst dst, const FFTPlan3D& p, size_t rows, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  {
    KTimer kt(KC_FFT_ROWS, st, (double)rows * (p.M * io_bytes<Src>() + (p.M + 1) * io_bytes<Dst>()));
    if (fs_split(p.M)) {
      if (launch_fs_r2c(src, dst, p.M, p.twm, p.twn, rows, st, &e)) {
        count_launch(1);
        return e;
      }
    }
  }
  return launch_r2c_rows_sh(src, dst, p, rows, st);
}

template <class Src, class Dst>
inline cudaError_t launch_c2r_rows(Src src, Dst dst, const FFTPlan3D& p, size_t rows, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  {
    KTimer kt(KC_FFT_ROWS, st, (double)rows * ((p.M + 1) * io_bytes<Src>() + p.M * io_bytes<Dst>()));
    if (fs_split(p.M)) {
      if (launch_fs_c2r(src, dst, p.M, p.twm, p.twn, rows, st, &e)) {
        count_launch(1);
        return e;
      }
    }
  }
  return launch_c2r_rows_sh(src, dst, p, rows, st);
}

// real [nx][ny][nz] -> half complex [nx][ny][nc] in `work`; the x pass
// writes through `xdst` (a CplxStore into work for a plain transform).
template <class RSrc, class XDst>
inline cudaError_t fft_r2c_3d(const FFTPlan3D& p, RSrc rsrc, float2* work, XDst xdst, cudaStream_t st) {
  cudaError_t e;
  const size_t rows = (size_t)p.nx * p.ny;
  e = launch_r2c_rows(rsrc, HalfStore{work, p.nc}, p, rows, st);
  if (e != cudaSuccess) return e;
  e = launch_strided(CplxLoad{work, p.ny, p.nc}, CplxStore{work, p.ny, p.nc}, p.py, p.twy, -1.f, p.nx, p.nc, st);
  if (e != cudaSuccess) return e;
  return launch_strided(CplxLoad{work, p.nx, p.ny * p.nc}, xdst, p.px, p.twx, -1.f, 1, p.ny * p.nc, st);
}

// half complex -> real; the x pass reads through `xsrc` (a CplxLoad, or a
// generator that synthesises the modes), `work` holds the intermediate.
template <class XSrc, class RDst>
inline cudaError_t fft_c2r_3d(const FFTPlan3D& p, XSrc xsrc, float2* work, RDst rdst, cudaStream_t st) {
  cudaError_t e;
  const size_t rows = (size_t)p.nx * p.ny;
  e = launch_strided(xsrc, CplxStore{work, p.nx, p.ny * p.nc}, p.px, p.twx, 1.f, 1, p.ny * p.nc, st);
  if (e != cudaSuccess) return e;
  e = launch_strided(CplxLoad{work, p.ny, p.nc}, CplxStore{work, p.ny, p.nc}, p.py, p.twy, 1.f, p.nx, p.nc, st);
  if (e != cudaSuccess) return e;
  return launch_c2r_rows(HalfLoad{work, p.nc}, rdst, p, rows, st);
}

}  // namespace exh
