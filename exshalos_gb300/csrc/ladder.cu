// FFT top-hat smoothing ladder and per-cell first-crossing map.
//
// For n_radii radii R_i log-spaced from one cell to R_max, the field is
// smoothed with the top-hat window W(kR) = 3 (sin x - x cos x) / x^3
// (exshalos_h.c:35-40) by one inverse FFT per radius, and each cell records
// the largest radius at which the smoothed density reaches the excursion-set
// barrier B(sigma^2(R)) (find_halos.c:4-44, 200-212): the first crossing when
// the ladder is walked from large to small scales.  255 = never crossed.
//
// The Fourier modes are generated once (the same Philox modes as the field)
// and read by the first pass of every radius; the barrier test and the map
// update run in the epilogue of the last pass, so no smoothed field is ever
// stored.
#include <cmath>
#include <string>
#include <vector>

#include "ctx.cuh"
#include "fft4.cuh"
#include "field.cuh"
#include "lpt.cuh"
#include "setup.h"

namespace exh {

__global__ void k_store_modes(FieldModes m, float2* __restrict__ out) {
  const size_t nk = (size_t)m.n0 * m.n1 * m.nc;
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; t < nk; t += stride) {
    const int k = (int)(t % m.nc);
    const size_t r = t / m.nc;
    out[t] = m.mode((int)(r / m.n1), (int)(r % m.n1), k);
  }
}

// W(k R) = 3 (sin x - x cos x) / x^3 (exshalos_h.c:35-40) for every radius
// and every integer |n|^2 of a cubic box, k = kf |n|: computed once per
// (box, radii) in FP64, where the difference s - x c loses no digits to
// cancellation at small x, and rounded to float.
__global__ void k_ladder_wtab(const float* __restrict__ R, int nr, int nn, double kf, float* __restrict__ w) {
  const size_t total = (size_t)nr * nn;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / nn), n2 = (int)(t % nn);
    const double x = kf * sqrt((double)n2) * (double)R[r];
    double v;
    if (x < 1e-3) {
      const double x2 = x * x;
      v = 1.0 - x2 * (0.1 - x2 * (1.0 / 280.0));
    } else {
      double sn, cs;
      sincos(x, &sn, &cs);
      v = 3.0 * (sn - x * cs) / (x * x * x);
    }
    w[t] = (float)v;
  }
}


// y-pass source (the y transform runs first): stored modes times W(|k| R);
// its tiles read runs of kz within one x plane, a better DRAM pattern than
// the x pass's planes 2 nd nc bytes apart
struct LadderGenY {
  static constexpr int io_bytes = 8;
  const float2* __restrict__ dk;
  const float* __restrict__ w;
  int n0, nc, h;
  __device__ __forceinline__ float2 operator()(int o, int e, int k) const {
    const int ii = (2 * o < n0) ? o : o - n0;
    const int jj = (2 * e < n0) ? e : e - n0;
    const int kk = (k == h) ? -h : k;
    const float wv = __ldg(&w[ii * ii + jj * jj + kk * kk]);
    const float2 v = dk[((size_t)o * n0 + e) * nc + k];
    return make_float2(v.x * wv, v.y * wv);
  }
};

// y pass of one radius for boxes with a four-step split of ny: the block's
// tile (x row o, W columns k0..k0+W-1, all n rows j) is multiplied by the
// window before the transform.  The W(|k| R) values it needs, one per
// (|j|, column), are gathered once from the |n|^2 table into shared memory
// (n/2 + 1 rows of W floats); a gather per element costs the pass about as
// much again as its loads of the modes.  The transform is the one of
// k_fft4_strided, so results equal the generic pass with LadderGenY.
template <int N1, int N2>
__global__ void __launch_bounds__(FS_THREADS, 4)
k_ladder_y(const float2* __restrict__ dk, const float* __restrict__ w, int h, float2* __restrict__ out,
           const float2* __restrict__ tw, int nc) {
  using S = FsShape<N1, N2>;
  constexpr int W = S::W, n = S::n, HJ = n / 2 + 1;
  __shared__ float2 sm[n * W];
  __shared__ float slab[HJ * W];
  const int o = blockIdx.y, i0 = blockIdx.x * W;
  const int nb = min(W, nc - i0);
  const int c = threadIdx.x % W, jj = threadIdx.x / W;
  const int ai = (2 * o < n) ? o : n - o;              // |i| of this x row (cubic box)
  for (int t = threadIdx.x; t < HJ * W; t += FS_THREADS) {
    const int aj = t / W, k = min(i0 + t % W, h);     // k <= h is |k|
    slab[t] = __ldg(&w[ai * ai + aj * aj + k * k]);
  }
  float2 v[N1];
  if (jj < N2) {
#pragma unroll
    for (int j1 = 0; j1 < N1; j1++)
      v[j1] = (c < nb) ? dk[((size_t)o * n + jj + N2 * j1) * nc + i0 + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  if (jj < N2) {
#pragma unroll
    for (int j1 = 0; j1 < N1; j1++) {
      const int e = jj + N2 * j1, aj = (2 * e < n) ? e : n - e;
      const float wv = slab[aj * W + c];
      v[j1] = make_float2(v[j1].x * wv, v[j1].y * wv);
    }
    RDft<N1>::run(v, 1.f, [tw](int m) { return __ldg(&tw[m * N2]); });
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) {
      float2 x = v[k1];
      if (k1 != 0 && jj != 0) x = cmul(x, tw_get(tw, jj * k1, 1.f));
      sm[(k1 * N2 + jj) * W + c] = x;
    }
  }
  __syncthreads();
  if (jj < N1) {
    float2 u[N2];
#pragma unroll
    for (int j2 = 0; j2 < N2; j2++) u[j2] = sm[(jj * N2 + j2) * W + c];
    RDft<N2>::run(u, 1.f, [tw](int m) { return __ldg(&tw[m * N1]); });
    if (c < nb) {
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) out[((size_t)o * n + jj + N1 * k2) * nc + i0 + c] = u[k2];
    }
  }
}

// launches k_ladder_y when ny has a four-step split; false otherwise
static bool launch_ladder_y(const FFTPlan3D& p, const float2* dk, const float* w, int h, float2* out,
                            cudaStream_t st, cudaError_t* err) {
  if (p.nx != p.ny || p.ny != p.nz) return false;     // the slab indexes x, y and z alike
  switch (fs_split(p.ny)) {
#define X(A_, B_)                                                                                      \
  case A_ * 1000 + B_: {                                                                               \
    constexpr int W_ = FsShape<A_, B_>::W;                                                             \
    KTimer kt(KC_FFT_STRIDED, st, (double)p.ny * p.nc * p.nx * 16.0);                                  \
    k_ladder_y<A_, B_><<<dim3(exh_div_up(p.nc, W_), p.nx), FS_THREADS, 0, st>>>(dk, w, h, out, p.twy, p.nc); \
    count_launch(1);                                                                                   \
    *err = cudaGetLastError();                                                                         \
    return true;                                                                                       \
  }
    EXH_FS_CASES(X)
#undef X
    default: return false;
  }
}

// z-pass destination: barrier test, first crossing kept
struct CrossStore {
  static constexpr int io_bytes = 4;     // two u8 reads and writes per pair
  unsigned char* __restrict__ cross;
  int N;
  float normx, B;
  int r;
  __device__ __forceinline__ void operator()(size_t row, int m, float2 v) const {
    unsigned char* c = cross + row * N + 2 * m;
    const unsigned char c0 = c[0], c1 = c[1];
    if (c0 == 255 && v.x * normx >= B) c[0] = (unsigned char)r;
    if (c1 == 255 && v.y * normx >= B) c[1] = (unsigned char)r;
  }
};

// z pass of one radius with the barrier test, for boxes whose block tile of
// the u8 map (R rows of 2M bytes) is a whole number of 16-byte chunks per
// thread: the block's map bytes are loaded at the start, with the row data,
// and written back once as 16-byte vectors after the transform.
template <int N1, int N2>
__global__ void __launch_bounds__(FS_THREADS)
k_ladder_z(const float2* __restrict__ work, const float2* __restrict__ twM, const float2* __restrict__ twN,
           unsigned char* __restrict__ cross, float normx, float B, int r) {
  using S = FsShape<N1, N2>;
  constexpr int M = S::n, R = S::R, LDA = FsRows<N1, N2>::LDA, nc = M + 1;
  constexpr int CHUNKS = (R * 2 * M) / (16 * FS_THREADS);      // 16-byte chunks per thread
  static_assert(CHUNKS >= 1 && (R * 2 * M) % (16 * FS_THREADS) == 0, "tile of whole 16-byte chunks");
  extern __shared__ float2 x[];                    // 2 * R * LDA
  float2* a = x + R * LDA;
  const size_t r0 = (size_t)blockIdx.x * R;
  uint4* tile = reinterpret_cast<uint4*>(cross + r0 * (2 * M));
  uint4 cm[CHUNKS];
#pragma unroll
  for (int q = 0; q < CHUNKS; q++) cm[q] = tile[threadIdx.x + q * FS_THREADS];
#pragma unroll
  for (int t = threadIdx.x; t < R * nc; t += FS_THREADS) {
    const int b = t / nc, k = t % nc;
    float2 v = work[(r0 + b) * nc + k];
    if (k == 0 || k == M) v.y = 0.f;
    x[b * LDA + k] = v;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < R * M; t += FS_THREADS) {
    const int b = t / M, k = t % M;
    const float2 xk = x[b * LDA + k];
    const float2 xm = cconj(x[b * LDA + (M - k)]);
    const float2 d = cmul(tw_get(twN, k, 1.f), csub(xk, xm));
    a[b * LDA + k] = make_float2(xk.x + xm.x - d.y, xk.y + xm.y + d.x);
  }
  __syncthreads();
  fs_rows_smem<N1, N2>(a, LDA, twM, 1.f);
  const unsigned char rb = (unsigned char)r;
#pragma unroll
  for (int q = 0; q < CHUNKS; q++) {
    const int o = (threadIdx.x + q * FS_THREADS) * 16;          // byte offset in the tile
    const int b = o / (2 * M), m0 = (o % (2 * M)) / 2;
    unsigned w[4] = {cm[q].x, cm[q].y, cm[q].z, cm[q].w};
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const float2 v = a[b * LDA + m0 + i];
      const int s0 = (2 * i) & 3, wi = (2 * i) >> 2;             // bytes 2i and 2i+1 of the chunk
      unsigned c0 = (w[wi] >> (8 * s0)) & 0xFFu, c1 = (w[wi] >> (8 * (s0 + 1))) & 0xFFu;
      if (c0 == 255u && v.x * normx >= B) c0 = rb;
      if (c1 == 255u && v.y * normx >= B) c1 = rb;
      w[wi] = (w[wi] & ~(0xFFFFu << (8 * s0))) | (c0 << (8 * s0)) | (c1 << (8 * (s0 + 1)));
    }
    tile[threadIdx.x + q * FS_THREADS] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// z pass of one radius for nz = 256 (M = 128 packed complex values per row),
// one warp per row and no shared memory.  Lane l holds the half-complex
// values k = l + 32 j (j < 4); the c2r pre-processing pairs k with M - k,
// which sits in lane (32 - l) mod 32, register 3 - j (lane 0 keeps its own).
// The inverse 128-point DFT of the packed rows is a 4-point DFT in registers
// (n = l + 32 n1), the twiddles w_128^(l m1), then a 32-point DFT across the
// lanes by five radix-2 decimation-in-frequency stages with shfl_xor.  Lane l
// then holds outputs m1 + 4 bitrev5(l), i.e. the eight consecutive reals
// 8 bitrev5(l) .. + 7 of the row, whose eight crossing-map bytes it updates
// with one 8-byte load and store.  Two rows per warp for more loads in flight.
__device__ __forceinline__ float2 shfl_c(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ float2 shfl_xor_c(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

constexpr int LZ_ROWS = 2;      // rows per warp

__global__ void __launch_bounds__(256)
k_ladder_z128(const float2* __restrict__ work, const float2* __restrict__ twM, const float2* __restrict__ twN,
              unsigned char* __restrict__ cross, size_t rows, float normx, float B, int r) {
  constexpr int nc = 129, RW = LZ_ROWS;
  const int lane = threadIdx.x & 31;
  const size_t row0 = ((size_t)blockIdx.x * 8 + (threadIdx.x >> 5)) * RW;
  if (row0 >= rows) return;                           // rows % RW == 0: whole warps leave
  float2 X[RW][4], XM[RW];
#pragma unroll
  for (int q = 0; q < RW; q++) {
    const float2* x = work + (row0 + q) * nc;
#pragma unroll
    for (int j = 0; j < 4; j++) X[q][j] = x[lane + 32 * j];
    XM[q] = lane == 0 ? x[128] : make_float2(0.f, 0.f);
    if (lane == 0) { X[q][0].y = 0.f; XM[q].y = 0.f; }   // k = 0 and k = M are real
  }
  const int pl = (32 - lane) & 31;
  float2 tN[4];
#pragma unroll
  for (int j = 0; j < 4; j++) tN[j] = tw_get(twN, lane + 32 * j, 1.f);
  float2 Y[RW][4];
#pragma unroll
  for (int q = 0; q < RW; q++) {
    float2 a[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      float2 xm = shfl_c(X[q][3 - j], pl);
      if (lane == 0) xm = (j == 0) ? XM[q] : X[q][(4 - j) & 3];
      xm = cconj(xm);
      const float2 d = cmul(tN[j], csub(X[q][j], xm));
      a[j] = make_float2(X[q][j].x + xm.x - d.y, X[q][j].y + xm.y + d.x);
    }
    const float2 s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]), s13 = cadd(a[1], a[3]), d13 = csub(a[1], a[3]);
    Y[q][0] = cadd(s02, s13);
    Y[q][2] = csub(s02, s13);
    Y[q][1] = make_float2(d02.x - d13.y, d02.y + d13.x);     // d02 + i d13
    Y[q][3] = make_float2(d02.x + d13.y, d02.y - d13.x);     // d02 - i d13
  }
#pragma unroll
  for (int m1 = 1; m1 < 4; m1++) {
    const float2 w = tw_get(twM, lane * m1, 1.f);
#pragma unroll
    for (int q = 0; q < RW; q++) Y[q][m1] = cmul(Y[q][m1], w);
  }
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool hi = (lane & h) != 0;
    const float2 w = tw_get(twM, (lane & (h - 1)) * (64 / h), 1.f);    // w_(2h)^(l mod h)
#pragma unroll
    for (int q = 0; q < RW; q++)
#pragma unroll
      for (int m1 = 0; m1 < 4; m1++) {
        const float2 pv = shfl_xor_c(Y[q][m1], h);
        Y[q][m1] = hi ? cmul(csub(pv, Y[q][m1]), w) : cadd(Y[q][m1], pv);
      }
  }
  const int br = (int)(__brev((unsigned)lane) >> 27);
  const unsigned long long rb = (unsigned long long)(unsigned char)r;
#pragma unroll
  for (int q = 0; q < RW; q++) {
    unsigned long long* cp = reinterpret_cast<unsigned long long*>(cross + (row0 + q) * 256 + 8 * br);
    unsigned long long mw = *cp;
    const float v[8] = {Y[q][0].x, Y[q][0].y, Y[q][1].x, Y[q][1].y, Y[q][2].x, Y[q][2].y, Y[q][3].x, Y[q][3].y};
#pragma unroll
    for (int b = 0; b < 8; b++) {
      const unsigned c = (unsigned)(mw >> (8 * b)) & 0xFFu;
      if (c == 255u && v[b] * normx >= B) mw = (mw & ~(0xFFull << (8 * b))) | (rb << (8 * b));
    }
    *cp = mw;
  }
}

// launches k_ladder_z when the box has a tile split for it; false otherwise
static bool launch_ladder_z(const FFTPlan3D& p, const float2* work, unsigned char* cross, float normx, float B, int r,
                            cudaStream_t st, cudaError_t* err) {
  const size_t rows = (size_t)p.nx * p.ny;
  if (reinterpret_cast<uintptr_t>(cross) % 16) return false;     // 16-byte vectors need an aligned map
  if (p.M == 128 && rows % (8 * LZ_ROWS) == 0) {
    KTimer kt(KC_FFT_ROWS, st, (double)rows * (129 * 8.0 + 256 * 2.0));
    k_ladder_z128<<<(unsigned)(rows / (8 * LZ_ROWS)), 256, 0, st>>>(work, p.twm, p.twn, cross, rows, normx, B, r);
    count_launch(1);
    *err = cudaGetLastError();
    return true;
  }
  switch (fs_split(p.M)) {
#define X(A_, B_)                                                                                      \
  case A_ * 1000 + B_: {                                                                               \
    constexpr int R_ = FsShape<A_, B_>::R, M_ = A_ * B_;                                               \
    if constexpr ((R_ * 2 * M_) % (16 * FS_THREADS) == 0) {                                            \
      if (rows % R_) return false;                                                                     \
      const size_t sm = 2 * sizeof(float2) * R_ * FsRows<A_, B_>::LDA;                                \
      *err = set_smem(k_ladder_z<A_, B_>, sm);                                                         \
      if (*err != cudaSuccess) return true;                                                            \
      KTimer kt(KC_FFT_ROWS, st, (double)rows * ((M_ + 1) * 8.0 + M_ * 4.0));                          \
      k_ladder_z<A_, B_><<<(unsigned)(rows / R_), FS_THREADS, sm, st>>>(work, p.twm, p.twn, cross, normx, B, r); \
      count_launch(1);                                                                                 \
      *err = cudaGetLastError();                                                                       \
      return true;                                                                                     \
    }                                                                                                  \
    return false;                                                                                      \
  }
    EXH_FS_CASES(X)
#undef X
    default: return false;
  }
}

int smoothing_ladder(Ctx& c, const BoxParams& b, const FieldModes& modes, int n_radii, const float* R,
                     const float* B, unsigned char* cross, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
  const size_t nk = (size_t)b.nd[0] * b.nd[1] * p->nc;
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  EXH_TRY(c.buf[B_LADDER].ensure(sizeof(float2) * nk));
  float2* work = c.buf[B_WORK].as<float2>();
  float2* dk = c.buf[B_LADDER].as<float2>();
  {
    KTimer kt(KC_OTHER, st, 8.0 * nk);
    k_store_modes<<<EXH_NUM_SMS * 16, 256, 0, st>>>(modes, dk);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  // window table, reused while the box and the radii repeat
  const int h = b.nd[0] / 2, nn = 3 * h * h + 1;
  std::string key(reinterpret_cast<const char*>(b.nd), sizeof(b.nd));
  key.append(reinterpret_cast<const char*>(&b.Lc), sizeof(float));
  key.append(reinterpret_cast<const char*>(R), sizeof(float) * n_radii);
  EXH_TRY(c.buf[B_LADDERW].ensure(sizeof(float) * ((size_t)n_radii * nn + n_radii)));
  float* wtab = c.buf[B_LADDERW].as<float>();
  if (key != c.ladder_key) {
    c.ladder_key.clear();
    float* dR = wtab + (size_t)n_radii * nn;
    EXH_CUDA_TRY(cudaMemcpyAsync(dR, R, sizeof(float) * n_radii, cudaMemcpyHostToDevice, st));
    const double kf = 2.0 * M_PI / ((double)b.Lc * b.nd[0]);
    KTimer kt(KC_OTHER, st, 4.0 * n_radii * nn);
    k_ladder_wtab<<<EXH_NUM_SMS * 8, 256, 0, st>>>(dR, n_radii, nn, kf, wtab);
    count_launch(1);
    const cudaError_t le = cudaGetLastError();
    // the copy reads host memory that the next call may reassign: wait for
    // it before returning, also when the launch failed
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    EXH_CUDA_TRY(le);
    c.ladder_key = key;
  }
  EXH_CUDA_TRY(cudaMemsetAsync(cross, 255, b.ng, st));
  // the radius loop: y then x (both complex, in either order), then the z
  // pass with the barrier test; the mode read and the window sit in the y
  // pass.  Three kernels per radius, the same sequence whenever the buffers,
  // tables and map repeat.
  auto radii = [&](cudaStream_t s) -> int {
    for (int i = n_radii - 1; i >= 0; i--) {       // large scales first
      CrossStore cs{cross, b.nd[2], b.Normx, B[i], i};
      cudaError_t ey = cudaSuccess;
      if (!launch_ladder_y(*p, dk, wtab + (size_t)i * nn, h, work, s, &ey))
        ey = launch_strided(LadderGenY{dk, wtab + (size_t)i * nn, b.nd[0], p->nc, h}, CplxStore{work, p->ny, p->nc},
                            p->py, p->twy, 1.f, p->nx, p->nc, s);
      EXH_CUDA_TRY(ey);
      EXH_CUDA_TRY(launch_strided(CplxLoad{work, p->nx, p->ny * p->nc}, CplxStore{work, p->nx, p->ny * p->nc},
                                  p->px, p->twx, 1.f, 1, p->ny * p->nc, s));
      cudaError_t e = cudaSuccess;
      if (!launch_ladder_z(*p, work, cross, b.Normx, B[i], i, s, &e))
        e = launch_c2r_rows(HalfLoad{work, p->nc}, cs, *p, (size_t)p->nx * p->ny, s);
      EXH_CUDA_TRY(e);
    }
    return EXH_OK;
  };
  // With per-kernel timing on, the kernels are launched one by one.  Else
  // the loop is captured into a CUDA graph on the second call with the same
  // arguments (the first one settles buffers and kernel attributes) and
  // replayed with one launch from then on.
  if (timing_on()) return radii(st);
  std::string gk;
  const void* ptrs[5] = {p, dk, work, wtab, cross};
  gk.append(reinterpret_cast<const char*>(ptrs), sizeof(ptrs));
  gk.append(reinterpret_cast<const char*>(B), sizeof(float) * n_radii);
  gk.append(reinterpret_cast<const char*>(&b.Normx), sizeof(float));
  gk.append(reinterpret_cast<const char*>(b.nd), sizeof(b.nd));
  gk.append(c.ladder_key);
  if (c.ladder_graph && gk == c.ladder_graph_key) {
    EXH_CUDA_TRY(cudaGraphLaunch(c.ladder_graph, st));
    count_launch(3 * n_radii);
    return EXH_OK;
  }
  if (gk != c.ladder_seen_key) {
    c.ladder_seen_key = gk;
    return radii(st);
  }
  cudaStream_t cap;
  EXH_TRY(c.side_stream(&cap));
  EXH_CUDA_TRY(cudaStreamSynchronize(cap));
  EXH_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  const int rs = radii(cap);
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(cap, &g);
  cudaGraphExec_t ex = nullptr;
  if (rs == EXH_OK && ec == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
    cudaGraphDestroy(g);
    if (c.ladder_graph) cudaGraphExecDestroy(c.ladder_graph);
    c.ladder_graph = ex;
    c.ladder_graph_key = gk;
    EXH_CUDA_TRY(cudaGraphLaunch(ex, st));        // the captured kernels were counted once when captured
    return EXH_OK;
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();                              // capture not possible: launch directly
  return radii(st);
}

}  // namespace exh

using namespace exh;

extern "C" int exh_smoothing_ladder(exh_ctx* ctx, const float* k, const float* P, int Nk, const exh_halo_params* prm,
                                    int n_radii, float R_max, uint8_t* cross, float* radii_out, float* barrier_out,
                                    int mem, void* stream) {
  if (!ctx || !k || !P || !prm || !cross) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  BoxParams b;
  EXH_TRY(setup_box(&b, prm->ndx, prm->ndy, prm->ndz, prm->Lc, prm->Om0, prm->redshift, prm->dc, prm->Nmin, prm->a,
                    prm->beta, prm->alpha, prm->seed));
  // radii and barriers, reused while every input they depend on repeats
  std::string key(reinterpret_cast<const char*>(k), sizeof(float) * (size_t)std::max(Nk, 0));
  key.append(reinterpret_cast<const char*>(P), sizeof(float) * (size_t)std::max(Nk, 0));
  const float kf[9] = {R_max, b.Lc, b.dc, b.Omz, b.a, b.beta, b.alpha, (float)n_radii, (float)b.DO_EB};
  key.append(reinterpret_cast<const char*>(kf), sizeof(kf));
  if (key != c.ladder_tab_key) {
    c.ladder_tab_key.clear();
    if (ladder_tables(b, k, P, Nk, n_radii, R_max, c.ladder_R, c.ladder_B) != EXH_OK) {
      exh_set_error_msg("ladder needs 1..255 radii and R_max >= Lc", __FILE__, __LINE__);
      return EXH_E_INVALID;
    }
    c.ladder_tab_key = key;
  }
  const std::vector<float>& R = c.ladder_R;
  const std::vector<float>& B = c.ladder_B;
  float* A_dev = nullptr;
  EXH_TRY(upload_amplitudes(c, b, k, P, Nk, &A_dev, st));
  FieldModes modes;
  EXH_TRY(make_field_modes(c, b, A_dev, prm->field_stream, prm->fixed, prm->phase, st, &modes));
  unsigned char* out = reinterpret_cast<unsigned char*>(cross);
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_CROSS].ensure(b.ng));
    out = c.buf[B_CROSS].as<unsigned char>();
  }
  EXH_TRY(smoothing_ladder(c, b, modes, n_radii, R.data(), B.data(), out, st));
  if (mem == EXH_MEM_HOST) {
    EXH_CUDA_TRY(cudaMemcpyAsync(cross, out, b.ng, cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    EXH_TRY(taus_verify(c));
  }
  // a device map is complete when `stream` reaches this point (no host wait)
  for (int i = 0; i < n_radii; i++) {
    if (radii_out) radii_out[i] = R[i];
    if (barrier_out) barrier_out[i] = B[i];
  }
  return EXH_OK;
}
