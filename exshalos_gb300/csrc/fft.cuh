// Shared-memory Stockham FFTs for sm_103a.
//
// A 3-D real transform (FFTW conventions: unnormalised, forward sign -1,
// half-complex last axis of nz/2+1 bins) runs as three HBM passes:
//   z: rows of nz reals <-> nz/2+1 bins (half-length complex FFT + split),
//   y, x: strided complex columns, tiles of W adjacent columns.
// Each pass stages a tile in shared memory and runs the mixed-radix (8,4,2,3)
// Stockham autosort network there (Govindaraju et al., SC'08 formulation),
// so no bit-reversal pass is needed.  Passes take source/destination
// functors, which lets producers (field synthesis, Poisson kernels) and
// consumers (P(k) binning, barrier tests) run inside the first or last pass
// instead of as separate sweeps over HBM.
#pragma once
#include "exh_common.cuh"
#include "timing.cuh"

namespace exh {

struct RadixPlan {
  int n;
  int nst;
  int r[12];
};

constexpr int FFT_THREADS = 256;
constexpr int FFT_W = 16;          // columns per strided tile: 16 x 8 B = 128 B rows
constexpr int FFT_ROWS = 16;       // rows per contiguous-axis tile
constexpr int FFT_LDB = FFT_ROWS + 1;

__device__ __forceinline__ float2 tw_get(const float2* __restrict__ tw, int m, float sgn) {
  float2 t = __ldg(&tw[m]);
  return make_float2(t.x, sgn * t.y);
}
__device__ __forceinline__ float2 mul_i(float2 a, float sgn) {  // a * (sgn * i)
  return make_float2(-sgn * a.y, sgn * a.x);
}

template <int R> __device__ __forceinline__ void dft(float2* v, float sgn);

template <> __device__ __forceinline__ void dft<2>(float2* v, float) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
template <> __device__ __forceinline__ void dft<3>(float2* v, float sgn) {
  const float s3 = 0.86602540378443864676f;
  float2 a = v[0], t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
  float2 m = make_float2(a.x - 0.5f * t1.x, a.y - 0.5f * t1.y);
  float2 r = mul_i(cscale(t2, s3), sgn);
  v[0] = cadd(a, t1);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}
template <> __device__ __forceinline__ void dft<4>(float2* v, float sgn) {
  float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  float2 t2 = cadd(v[1], v[3]), t3 = mul_i(csub(v[1], v[3]), sgn);
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}
template <> __device__ __forceinline__ void dft<8>(float2* v, float sgn) {
  const float h = 0.70710678118654752440f;
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  dft<4>(e, sgn);
  dft<4>(o, sgn);
  float2 w1 = make_float2(h, sgn * h), w3 = make_float2(-h, sgn * h);
  float2 o1 = cmul(o[1], w1), o2 = mul_i(o[2], sgn), o3 = cmul(o[3], w3);
  v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], o1);   v[5] = csub(e[1], o1);
  v[2] = cadd(e[2], o2);   v[6] = csub(e[2], o2);
  v[3] = cadd(e[3], o3);   v[7] = csub(e[3], o3);
}

// One Stockham stage over nb transforms of length n held column-wise in
// shared memory: element e of transform b at [e * ldb + b].
template <int R>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ in, float2* __restrict__ out,
                                               int n, int Ns, int nb, int ldb,
                                               const float2* __restrict__ tw, float sgn) {
  const int nbf = n / R, total = nbf * nb, step = n / (Ns * R);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int b = t % nb, j = t / nb, k = j % Ns;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = in[(j + r * nbf) * ldb + b];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], tw_get(tw, r * k * step, sgn));
    }
    dft<R>(v, sgn);
    const int d = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) out[(d + r * Ns) * ldb + b] = v[r];
  }
}

// Runs every stage; a and b are ping-pong buffers, returns the one holding
// the result.  Synchronises the block before returning.
__device__ __forceinline__ float2* stockham_run(float2* a, float2* b, const RadixPlan& pl, int nb, int ldb,
                                                const float2* __restrict__ tw, float sgn) {
  int Ns = 1;
  for (int s = 0; s < pl.nst; s++) {
    const int R = pl.r[s];
    if (R == 8) stockham_stage<8>(a, b, pl.n, Ns, nb, ldb, tw, sgn);
    else if (R == 4) stockham_stage<4>(a, b, pl.n, Ns, nb, ldb, tw, sgn);
    else if (R == 2) stockham_stage<2>(a, b, pl.n, Ns, nb, ldb, tw, sgn);
    else stockham_stage<3>(a, b, pl.n, Ns, nb, ldb, tw, sgn);
    __syncthreads();
    float2* t = a; a = b; b = t;
    Ns *= R;
  }
  return a;
}

// ---------------------------------------------------------------- functors
// complex array [outer][n][inner]
struct CplxLoad {
  static constexpr int io_bytes = 8;
  const float2* __restrict__ p;
  int n, inner;
  __device__ __forceinline__ float2 operator()(int o, int e, int i) const {
    return p[((size_t)o * n + e) * inner + i];
  }
};
struct CplxStore {
  static constexpr int io_bytes = 8;
  float2* __restrict__ p;
  int n, inner;
  __device__ __forceinline__ void operator()(int o, int e, int i, float2 v) const {
    p[((size_t)o * n + e) * inner + i] = v;
  }
};
// real rows: element (row, m) of the packed pair view (x[2m], x[2m+1])
struct RealPairLoad {
  static constexpr int io_bytes = 8;
  const float* __restrict__ p;
  int N;
  __device__ __forceinline__ float2 operator()(size_t row, int m) const {
    return *reinterpret_cast<const float2*>(p + row * N + 2 * m);
  }
};
struct RealPairStore {
  static constexpr int io_bytes = 8;
  float* __restrict__ p;
  int N;
  float scale;
  __device__ __forceinline__ void operator()(size_t row, int m, float2 v) const {
    *reinterpret_cast<float2*>(p + row * N + 2 * m) = make_float2(v.x * scale, v.y * scale);
  }
};
// half-complex rows [row][nc]
struct HalfLoad {
  static constexpr int io_bytes = 8;
  const float2* __restrict__ p;
  int nc;
  __device__ __forceinline__ float2 operator()(size_t row, int k) const { return p[row * nc + k]; }
};
struct HalfStore {
  static constexpr int io_bytes = 8;
  float2* __restrict__ p;
  int nc;
  __device__ __forceinline__ void operator()(size_t row, int k, float2 v) const { p[row * nc + k] = v; }
};

// ---------------------------------------------------------------- kernels
// Strided pass: transform along e for a tile of W adjacent inner columns.
template <class Src, class Dst>
__global__ void __launch_bounds__(FFT_THREADS)
k_fft_strided(Src src, Dst dst, RadixPlan pl, const float2* __restrict__ tw, float sgn, int inner) {
  extern __shared__ float2 smem[];
  const int n = pl.n;
  float2* b0 = smem;
  float2* b1 = smem + n * FFT_W;
  const int o = blockIdx.y, i0 = blockIdx.x * FFT_W;
  const int nb = min(FFT_W, inner - i0);
  for (int t = threadIdx.x; t < n * FFT_W; t += blockDim.x) {
    const int e = t / FFT_W, b = t % FFT_W;
    b0[e * FFT_W + b] = (b < nb) ? src(o, e, i0 + b) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* res = stockham_run(b0, b1, pl, FFT_W, FFT_W, tw, sgn);
  for (int t = threadIdx.x; t < n * FFT_W; t += blockDim.x) {
    const int e = t / FFT_W, b = t % FFT_W;
    if (b < nb) dst(o, e, i0 + b, res[e * FFT_W + b]);
  }
}

// z pass, real -> half complex.  pl: length M = N/2; twN: e^{2 pi i k/N}.
template <class Src, class Dst>
__global__ void __launch_bounds__(FFT_THREADS)
k_fft_r2c_rows(Src src, Dst dst, RadixPlan pl, const float2* __restrict__ twM,
               const float2* __restrict__ twN, size_t rows) {
  extern __shared__ float2 smem[];
  const int M = pl.n;
  float2* b0 = smem;
  float2* b1 = smem + M * FFT_LDB;
  const size_t r0 = (size_t)blockIdx.x * FFT_ROWS;
  const int nb = (int)min((size_t)FFT_ROWS, rows - r0);
  for (int t = threadIdx.x; t < M * FFT_ROWS; t += blockDim.x) {
    const int b = t / M, m = t % M;
    b0[m * FFT_LDB + b] = (b < nb) ? src(r0 + b, m) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* Z = stockham_run(b0, b1, pl, FFT_ROWS, FFT_LDB, twM, -1.f);
  const int nc = M + 1;
  for (int t = threadIdx.x; t < nc * FFT_ROWS; t += blockDim.x) {
    const int b = t / nc, k = t % nc;
    if (b >= nb) continue;
    const float2 zk = Z[(k == M ? 0 : k) * FFT_LDB + b];
    const float2 zm = cconj(Z[(k == 0 ? 0 : M - k) * FFT_LDB + b]);
    const float2 A = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y));
    const float2 d = csub(zk, zm);
    const float2 Bv = make_float2(0.5f * d.y, -0.5f * d.x);      // -i/2 (zk - zm)
    const float2 w = tw_get(twN, k, -1.f);                       // e^{-2 pi i k/N}
    dst(r0 + b, k, cadd(A, cmul(w, Bv)));
  }
}

// z pass, half complex -> real.  The imaginary parts of bins 0 and N/2 are
// ignored, as in a c2r transform of Hermitian data.
template <class Src, class Dst>
__global__ void __launch_bounds__(FFT_THREADS)
k_fft_c2r_rows(Src src, Dst dst, RadixPlan pl, const float2* __restrict__ twM,
               const float2* __restrict__ twN, size_t rows) {
  extern __shared__ float2 smem[];
  const int M = pl.n, nc = M + 1;
  float2* xs = smem;
  float2* b0 = smem + nc * FFT_LDB;
  float2* b1 = b0 + M * FFT_LDB;
  const size_t r0 = (size_t)blockIdx.x * FFT_ROWS;
  const int nb = (int)min((size_t)FFT_ROWS, rows - r0);
  for (int t = threadIdx.x; t < nc * FFT_ROWS; t += blockDim.x) {
    const int b = t / nc, k = t % nc;
    float2 v = (b < nb) ? src(r0 + b, k) : make_float2(0.f, 0.f);
    if (k == 0 || k == M) v.y = 0.f;
    xs[k * FFT_LDB + b] = v;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < M * FFT_ROWS; t += blockDim.x) {
    const int b = t % FFT_ROWS, k = t / FFT_ROWS;
    const float2 xk = xs[k * FFT_LDB + b];
    const float2 xm = cconj(xs[(M - k) * FFT_LDB + b]);
    const float2 w = tw_get(twN, k, 1.f);                        // e^{+2 pi i k/N}
    const float2 d = cmul(w, csub(xk, xm));
    b0[k * FFT_LDB + b] = make_float2(xk.x + xm.x - d.y, xk.y + xm.y + d.x);  // (xk+xm) + i d
  }
  __syncthreads();
  float2* z = stockham_run(b0, b1, pl, FFT_ROWS, FFT_LDB, twM, 1.f);
  for (int t = threadIdx.x; t < M * FFT_ROWS; t += blockDim.x) {
    const int b = t / M, m = t % M;
    if (b < nb) dst(r0 + b, m, z[m * FFT_LDB + b]);
  }
}

// ---------------------------------------------------------------- plans
struct FFTPlan3D {
  int nx = 0, ny = 0, nz = 0, nc = 0, M = 0;
  RadixPlan px{}, py{}, pm{};
  float2 *twx = nullptr, *twy = nullptr, *twm = nullptr, *twn = nullptr;
};

RadixPlan make_radix_plan(int n);   // fft.cu
int fft_plan_create(FFTPlan3D* p, int nx, int ny, int nz);
void fft_plan_destroy(FFTPlan3D* p);
void count_launch(int n);          // host-side launch counter (capi.cu)

// A small host-to-device upload (at most 256 bytes: counters, control
// blocks) carried as a kernel argument, so the bytes are captured when the
// launch is enqueued and the host source may change or go out of scope at
// once.  cudaMemcpyAsync from pageable memory does not promise that: where
// the GPU reads pageable memory directly, the copy may run later, from
// whatever the stack holds by then.  (fft.cu)
constexpr size_t UPLOAD_SMALL_MAX = 256;
int upload_small(void* dst, const void* src, size_t bytes, cudaStream_t st);

inline size_t smem_strided(int n) { return sizeof(float2) * 2 * (size_t)n * FFT_W; }
inline size_t smem_r2c(int M) { return sizeof(float2) * 2 * (size_t)M * FFT_LDB; }
inline size_t smem_c2r(int M) { return sizeof(float2) * (3 * (size_t)M + 1) * FFT_LDB; }

// Raise a kernel's dynamic shared-memory limit to at least `bytes`.  The
// attribute is process-wide while contexts on several host threads launch
// the same kernel with different sizes, so it only ever grows (under a lock,
// per device): lowering it for a small box could make another thread's
// launch for a larger one fail between its own call and its launch.
cudaError_t smem_raise(const void* kernel, size_t bytes);     // fft.cu

template <class K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
  return smem_raise(reinterpret_cast<const void*>(kernel), bytes);
}

// Strided pass launcher: data [outer][n][inner].
// bytes each functor moves per complex element (0 for generators)
template <class F> constexpr int io_bytes() { return F::io_bytes; }

template <class Src, class Dst>
inline cudaError_t launch_strided_sh(Src src, Dst dst, const RadixPlan& pl, const float2* tw, float sgn,
                                  int outer, int inner, cudaStream_t st) {
  auto kern = k_fft_strided<Src, Dst>;
  size_t sm = smem_strided(pl.n);
  cudaError_t e = set_smem(kern, sm);
  if (e != cudaSuccess) return e;
  dim3 grid(exh_div_up(inner, FFT_W), outer);
  KTimer kt(KC_FFT_STRIDED, st, (double)pl.n * inner * outer * (io_bytes<Src>() + io_bytes<Dst>()));
  kern<<<grid, FFT_THREADS, sm, st>>>(src, dst, pl, tw, sgn, inner);
  count_launch(1);
  return cudaGetLastError();
}

template <class Src, class Dst>
inline cudaError_t launch_r2c_rows_sh(Src src, Dst dst, const FFTPlan3D& p, size_t rows, cudaStream_t st) {
  auto kern = k_fft_r2c_rows<Src, Dst>;
  size_t sm = smem_r2c(p.M);
  cudaError_t e = set_smem(kern, sm);
  if (e != cudaSuccess) return e;
  KTimer kt(KC_FFT_ROWS, st, (double)rows * (p.M * io_bytes<Src>() + (p.M + 1) * io_bytes<Dst>()));
  kern<<<exh_div_up(rows, FFT_ROWS), FFT_THREADS, sm, st>>>(src, dst, p.pm, p.twm, p.twn, rows);
  count_launch(1);
  return cudaGetLastError();
}

template <class Src, class Dst>
inline cudaError_t launch_c2r_rows_sh(Src src, Dst dst, const FFTPlan3D& p, size_t rows, cudaStream_t st) {
  auto kern = k_fft_c2r_rows<Src, Dst>;
  size_t sm = smem_c2r(p.M);
  cudaError_t e = set_smem(kern, sm);
  if (e != cudaSuccess) return e;
  KTimer kt(KC_FFT_ROWS, st, (double)rows * ((p.M + 1) * io_bytes<Src>() + p.M * io_bytes<Dst>()));
  kern<<<exh_div_up(rows, FFT_ROWS), FFT_THREADS, sm, st>>>(src, dst, p.pm, p.twm, p.twn, rows);
  count_launch(1);
  return cudaGetLastError();
}

}  // namespace exh
