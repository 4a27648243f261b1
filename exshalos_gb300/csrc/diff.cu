// Differentiable forward model and its hand-written adjoint:
//
//   noise w (real, nd^3) -> W = r2c(w) -> delta_k = W sqrt(p(k) / nd^3),
//   p(k) log-linear in log k between knot amplitudes P_i
//   -> 1LPT: phi1 = c2r(-delta_k / k^2), S1 = -Normx D phi1   (lpt.c:11-96)
//   -> 2LPT: sigma = xx yy + xx zz + yy zz - xy^2 - xz^2 - yz^2 of D S1,
//      phi2 = c2r(r2c(sigma) Normk / (-k^2)), S2 = c2 Normx D phi2 (lpt.c:99-226)
//   -> particles x = q + S1 + S2 wrapped by cysumf (lpt.c:229-242)
//   -> CIC grid (gridmodule.c:21-53, 206-211) -> P(k) bins (powermodule.c:4-108)
//   -> chi^2 = sum_b (P_b - T_b)^2 / var_b, var_b = 2 T_b^2 / N_b by default.
//
// D is the sixth-order central difference of lpt.c:60-64 (stencil
// 1, -9, 45, 0, -45, 9, -1 over 60 Lc), whose adjoint is -D.  Unnormalised
// FFTs as FFTW: the adjoint of r2c is c2r of the gradient with the
// interior half-plane entries (0 < kz < nd/2) halved; the adjoint of c2r is
// r2c of the gradient with those entries doubled.  The forward keeps what
// the backward needs (W, the amplitudes, D S1, the particle positions and
// the transformed grid), so one forward serves one backward.
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "fft4.cuh"
#include "setup.h"
#include "spectrum.cuh"

namespace exh {

namespace {

constexpr int MAX_KNOTS = 64;

enum DiffBuf {
  DB_W = 0,    // r2c(noise), float2[nk]
  DB_A,        // amplitude per mode, float[nk]
  DB_WORK,     // complex work, float2[nk]
  DB_X,        // r2c(CIC grid), float2[nk]
  DB_PHI,      // phi1 / phi2 / gradient scratch, float[ng]
  DB_S1,       // S1 [3][ng]
  DB_D6,       // xx yy zz xy xz yz [6][ng]
  DB_SIG,      // sigma / gradient of sigma, float[ng]
  DB_POS,      // particles [ng][3]
  DB_GRID,     // CIC grid / its gradient, float[ng]
  DB_GS,       // gradient of S [3][ng]
  DB_G6,       // gradients of the six derivatives [6][ng]
  DB_GS1,      // gradient of S1 [3][ng]
  DB_GA,       // gradient of the amplitudes, float[nk]
  DB_BINS,     // per-block partials and per-bin tables
  DB_KNOTS,    // knots (log k, P) and their gradient partials
  DB_COUNT
};

struct KnotTab {
  int n;
  float lk[MAX_KNOTS];   // log k_i, increasing
  float P[MAX_KNOTS];
};

struct ModeGeom {
  int nd, nc, h;
  float kf;              // 2 pi / L
  __device__ __forceinline__ void at(size_t t, int& i, int& j, int& k, int& ii, int& jj, int& kk) const {
    k = (int)(t % nc);
    const size_t r = t / nc;
    j = (int)(r % nd);
    i = (int)(r / nd);
    ii = (2 * i < nd) ? i : i - nd;
    jj = (2 * j < nd) ? j : j - nd;
    kk = (k == h) ? -h : k;
  }
  __device__ __forceinline__ float k2(int ii, int jj, int kk) const {
    return kf * kf * (float)(ii * ii + jj * jj + kk * kk);
  }
};

// log-linear interpolation of p(k) in log k, constant beyond the end knots;
// returns p and the knot pair with its weights
__device__ __forceinline__ float knot_interp(const KnotTab& T, float lk, int& i0, float& t) {
  if (lk <= T.lk[0]) { i0 = 0; t = 0.f; return T.P[0]; }
  if (lk >= T.lk[T.n - 1]) { i0 = T.n - 2; t = 1.f; return T.P[T.n - 1]; }
  int lo = 0, hi = T.n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (T.lk[mid] > lk) hi = mid; else lo = mid;
  }
  i0 = lo;
  t = (lk - T.lk[lo]) / (T.lk[lo + 1] - T.lk[lo]);
  return expf((1.f - t) * logf(T.P[lo]) + t * logf(T.P[lo + 1]));
}

// ---------------------------------------------------------------- k space
// x pass of r2c(noise): keep W, the amplitude, and write phi1_k = -W A / k^2
struct NoiseStore {
  static constexpr int io_bytes = 20;
  float2* __restrict__ W;
  float* __restrict__ A;
  float2* __restrict__ work;
  ModeGeom g;
  KnotTab T;
  float inv_sqrt_ng;
  __device__ __forceinline__ void operator()(int, int e, int inner, float2 v) const {
    const size_t idx = (size_t)e * ((size_t)g.nd * g.nc) + inner;
    int i, j, k, ii, jj, kk;
    g.at(idx, i, j, k, ii, jj, kk);
    const float k2 = g.k2(ii, jj, kk);
    float a = 0.f, f = 0.f;
    if (k2 > 0.f) {
      int i0;
      float t;
      const float p = knot_interp(T, 0.5f * logf(k2), i0, t);
      a = sqrtf(p) * inv_sqrt_ng;
      f = -a / k2;
    }
    W[idx] = v;
    A[idx] = a;
    work[idx] = make_float2(v.x * f, v.y * f);
  }
};

// x pass of r2c: multiply by s / (-k^2) (0 at k = 0)
struct PoissonStore {
  static constexpr int io_bytes = 8;
  float2* __restrict__ out;
  ModeGeom g;
  float s;
  __device__ __forceinline__ void operator()(int, int e, int inner, float2 v) const {
    const size_t idx = (size_t)e * ((size_t)g.nd * g.nc) + inner;
    int i, j, k, ii, jj, kk;
    g.at(idx, i, j, k, ii, jj, kk);
    const float k2 = g.k2(ii, jj, kk);
    const float f = k2 > 0.f ? -s / k2 : 0.f;
    out[idx] = make_float2(v.x * f, v.y * f);
  }
};

// mode-skip rule and bin of powermodule.c:26-56 (reference float arithmetic);
// returns -1 when the mode is not binned, else the bin and the CIC factor
__device__ __forceinline__ int mode_bin(const BinParams& bp, int nd, int i, int j, int k, float& kmod, float& w) {
  if ((k == 0 || k == nd / 2) &&
      ((i > nd / 2 && j > nd / 2) || i == 0 || i == nd / 2 || j == 0 || j == nd / 2 || (i > nd / 2 && j < nd / 2)))
    return -1;
  const float kx = (float)((2 * i < nd) ? i : i - nd) * bp.kn;
  const float ky = (float)((2 * j < nd) ? j : j - nd) * bp.kn;
  const float kz = (float)((2 * k < nd) ? k : k - nd) * bp.kn;
  const float k2 = __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
  kmod = __fsqrt_rn(k2);
  const int bin = (int)floorf(__fdiv_rn(__fsub_rn(kmod, bp.kmin), bp.dk));
  if (bin < 0 || bin >= bp.Nk) return -1;
  auto sinc = [](float x) { return x != 0.f ? sinf(x) / x : 1.f; };
  w = sinc(kx * bp.Lb * 0.5f) * sinc(ky * bp.Lb * 0.5f) * sinc(kz * bp.Lb * 0.5f);
  w = w * w;
  return bin;
}

constexpr int BIN_T = 256;

// P(k) bins of the transformed CIC grid: per-block FP64 histograms
__global__ void __launch_bounds__(BIN_T)
k_diff_bin(const float2* __restrict__ X, size_t nk, int nd, int nc, BinParams bp, double* __restrict__ partP,
           double* __restrict__ partK, unsigned* __restrict__ partN) {
  extern __shared__ double hsm[];
  double* hP = hsm;
  double* hK = hP + bp.Nk;
  unsigned* hN = reinterpret_cast<unsigned*>(hK + bp.Nk);
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) { hP[b] = 0.0; hK[b] = 0.0; hN[b] = 0u; }
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nk; t += stride) {
    const int k = (int)(t % nc);
    const size_t r = t / nc;
    const int j = (int)(r % nd), i = (int)(r / nd);
    float kmod, w;
    const int bin = mode_bin(bp, nd, i, j, k, kmod, w);
    if (bin < 0) continue;
    const float2 v = X[t];
    const double s = (double)bp.Normk / (double)w;
    const double re = (double)v.x * s, im = (double)v.y * s;
    atomicAdd(&hP[bin], re * re + im * im);
    atomicAdd(&hK[bin], (double)kmod);
    atomicAdd(&hN[bin], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) {
    partP[(size_t)blockIdx.x * bp.Nk + b] = hP[b];
    partK[(size_t)blockIdx.x * bp.Nk + b] = hK[b];
    partN[(size_t)blockIdx.x * bp.Nk + b] = hN[b];
  }
}

__global__ void k_diff_bin_reduce(const double* __restrict__ partP, const double* __restrict__ partK,
                                  const unsigned* __restrict__ partN, int nblk, int Nk, double* __restrict__ out) {
  const int b = blockIdx.x;
  __shared__ double rP[256], rK[256];
  __shared__ unsigned long long rN[256];
  double sP = 0.0, sK = 0.0;
  unsigned long long sN = 0;
  for (int q = threadIdx.x; q < nblk; q += blockDim.x) {
    sP += partP[(size_t)q * Nk + b];
    sK += partK[(size_t)q * Nk + b];
    sN += partN[(size_t)q * Nk + b];
  }
  rP[threadIdx.x] = sP; rK[threadIdx.x] = sK; rN[threadIdx.x] = sN;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rP[threadIdx.x] += rP[threadIdx.x + s];
      rK[threadIdx.x] += rK[threadIdx.x + s];
      rN[threadIdx.x] += rN[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[3 * b] = rP[0];
    out[3 * b + 1] = rK[0];
    out[3 * b + 2] = (double)rN[0];
  }
}

// x-pass source of the backward c2r: dchi2/dX with the half-plane factor
struct BinGradLoad {
  static constexpr int io_bytes = 8;
  const float2* __restrict__ X;
  const float* __restrict__ gbin;   // 2 dchi2/dP_b / N_b per bin
  ModeGeom g;
  BinParams bp;
  __device__ __forceinline__ float2 operator()(int, int e, int inner) const {
    const size_t idx = (size_t)e * ((size_t)g.nd * g.nc) + inner;
    const int k = inner % g.nc, j = inner / g.nc;
    float kmod, w;
    const int bin = mode_bin(bp, g.nd, e, j, k, kmod, w);
    if (bin < 0) return make_float2(0.f, 0.f);
    const float s = bp.Normk / w;
    float f = gbin[bin] * s * s;
    if (k != 0 && k != g.h) f *= 0.5f;
    const float2 v = X[idx];
    return make_float2(v.x * f, v.y * f);
  }
};

// x pass of r2c(dchi2/dphi1): noise gradient source and amplitude gradient
struct NoiseGradStore {
  static constexpr int io_bytes = 28;
  const float2* __restrict__ W;
  const float* __restrict__ A;
  float2* __restrict__ work;
  float* __restrict__ gA;
  ModeGeom g;
  __device__ __forceinline__ void operator()(int, int e, int inner, float2 v) const {
    const size_t idx = (size_t)e * ((size_t)g.nd * g.nc) + inner;
    int i, j, k, ii, jj, kk;
    g.at(idx, i, j, k, ii, jj, kk);
    const float k2 = g.k2(ii, jj, kk);
    if (!(k2 > 0.f)) {
      work[idx] = make_float2(0.f, 0.f);
      gA[idx] = 0.f;
      return;
    }
    // d chi2 / d delta_k (stored entry, conjugate partner included)
    const float c = (k != 0 && k != g.h) ? 2.f : 1.f;
    const float f = -1.f / k2;
    const float2 gd = make_float2(c * f * v.x, c * f * v.y);
    const float2 w = W[idx];
    gA[idx] = w.x * gd.x + w.y * gd.y;
    // noise: c2r of the half-plane-weighted A * gd (the factors cancel)
    const float a = A[idx] * f;
    work[idx] = make_float2(a * v.x, a * v.y);
  }
};

// knot gradient: sum over modes of dchi2/dA dA/dP_i
__global__ void __launch_bounds__(BIN_T)
k_knot_grad(const float* __restrict__ gA, const float* __restrict__ A, size_t nk, ModeGeom g, KnotTab T,
            double* __restrict__ part) {
  __shared__ double h[MAX_KNOTS];
  for (int b = threadIdx.x; b < T.n; b += blockDim.x) h[b] = 0.0;
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nk; t += stride) {
    const float a = A[t];
    if (a == 0.f) continue;
    int i, j, k, ii, jj, kk;
    g.at(t, i, j, k, ii, jj, kk);
    int i0;
    float u;
    knot_interp(T, 0.5f * logf(g.k2(ii, jj, kk)), i0, u);
    // p = exp(l), l = (1-u) ln P_i0 + u ln P_i0+1;  dA/dP_i = A/2 dl/dP_i
    const double c = 0.5 * (double)gA[t] * (double)a;
    if (u < 1.f) atomicAdd(&h[i0], c * (1.0 - (double)u) / (double)T.P[i0]);
    if (u > 0.f) atomicAdd(&h[i0 + 1], c * (double)u / (double)T.P[i0 + 1]);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < T.n; b += blockDim.x) part[(size_t)blockIdx.x * T.n + b] = h[b];
}

__global__ void k_knot_reduce(const double* __restrict__ part, int nblk, int n, double* __restrict__ out) {
  const int b = blockIdx.x;
  __shared__ double r[256];
  double s = 0.0;
  for (int q = threadIdx.x; q < nblk; q += blockDim.x) s += part[(size_t)q * n + b];
  r[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) r[threadIdx.x] += r[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[b] = r[0];
}

// ---------------------------------------------------------------- real space
// raw sixth-order stencil along axis a (0 x, 1 y, 2 z) of f at (i, j, k)
__device__ __forceinline__ float fd6(const float* __restrict__ f, int a, int i, int j, int k, int nd) {
  auto at = [&](int s) {
    int ii = i, jj = j, kk = k;
    if (a == 0) ii = exh_wrap(i, s, nd);
    else if (a == 1) jj = exh_wrap(j, s, nd);
    else kk = exh_wrap(k, s, nd);
    return __ldg(&f[((size_t)ii * nd + jj) * nd + kk]);
  };
  return (at(3) - 9.f * at(2) + 45.f * at(1)) - (45.f * at(-1) - 9.f * at(-2) + at(-3));
}

__device__ __forceinline__ void cell_ijk(size_t c, int nd, int& i, int& j, int& k) {
  k = (int)(c % nd);
  const size_t r = c / nd;
  j = (int)(r % nd);
  i = (int)(r / nd);
}

// S1_a = s D_a phi (s = -Normx / (60 Lc))
__global__ void k_grad3(const float* __restrict__ phi, int nd, float s, float* __restrict__ S) {
  const size_t ng = (size_t)nd * nd * nd;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ng; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, nd, i, j, k);
#pragma unroll
    for (int a = 0; a < 3; a++) S[a * ng + c] = s * fd6(phi, a, i, j, k, nd);
  }
}

// the six derivatives of S1 and the second-order source (lpt.c:116-133)
__global__ void k_lpt2_src(const float* __restrict__ S, int nd, float inv60, float* __restrict__ d6,
                           float* __restrict__ sig) {
  const size_t ng = (size_t)nd * nd * nd;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ng; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, nd, i, j, k);
    const float xx = inv60 * fd6(S, 0, i, j, k, nd);
    const float xy = inv60 * fd6(S, 1, i, j, k, nd);
    const float xz = inv60 * fd6(S, 2, i, j, k, nd);
    const float yy = inv60 * fd6(S + ng, 1, i, j, k, nd);
    const float yz = inv60 * fd6(S + ng, 2, i, j, k, nd);
    const float zz = inv60 * fd6(S + 2 * ng, 2, i, j, k, nd);
    d6[c] = xx; d6[ng + c] = yy; d6[2 * ng + c] = zz;
    d6[3 * ng + c] = xy; d6[4 * ng + c] = xz; d6[5 * ng + c] = yz;
    sig[c] = xx * yy + xx * zz + yy * zz - xy * xy - xz * xz - yz * yz;
  }
}

// x = cysumf(q, S1 + s2 D phi2, L) (lpt.c:229-242, exshalos_h.c:13-21)
__global__ void k_particles(const float* __restrict__ S1, const float* __restrict__ phi2, int nd, float s2, float Lc,
                            float L, float* __restrict__ pos) {
  const size_t ng = (size_t)nd * nd * nd;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ng; c += (size_t)gridDim.x * blockDim.x) {
    int idx[3];
    cell_ijk(c, nd, idx[0], idx[1], idx[2]);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      float s = S1[a * ng + c];
      if (phi2) s += s2 * fd6(phi2, a, idx[0], idx[1], idx[2], nd);
      const float q = (float)((double)(idx[a] * Lc) + Lc / 2.0);
      float r = q + s;
      if (r >= L) r -= L;
      if (r < 0.f) r += L;
      pos[3 * c + a] = r;
    }
  }
}

// adjoint of the CIC assignment of k_cic: dchi2/dx of every particle
__global__ void k_cic_adjoint(const float* __restrict__ pos, size_t np, int nd, float L, float Ld, float scale,
                              const float* __restrict__ g, float* __restrict__ gS) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
    int lo[3], hi[3];
    float dx[3], t[3], sg[3];
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      float x = pos[3 * p + a];
      for (int it = 0; it < 64 && x >= L; it++) x = __fsub_rn(x, L);
      for (int it = 0; it < 64 && x < 0.f; it++) x = __fadd_rn(x, L);
      if (!(x >= 0.f && x < L)) ok = false;
      const float q = __fdiv_rn(x, Ld);
      int c = (int)floorf(q);
      if (c >= nd) c = nd - 1;
      float d = __fsub_rn(q, (float)c + 0.5f);
      int s = 1;
      if (d < 0.f) { s = -1; d = -d; }
      lo[a] = c;
      hi[a] = exh_wrap(c, s, nd);
      dx[a] = d;
      t[a] = 1.f - d;
      sg[a] = (float)s;
    }
    if (!ok) {
      gS[p] = 0.f; gS[np + p] = 0.f; gS[2 * np + p] = 0.f;
      continue;
    }
    const size_t n2 = (size_t)nd * nd;
    float gv[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int c = 0; c < 2; c++)
          gv[a][b][c] = __ldg(&g[(a ? hi[0] : lo[0]) * n2 + (size_t)(b ? hi[1] : lo[1]) * nd + (c ? hi[2] : lo[2])]);
    const float wy[2] = {t[1], dx[1]}, wz[2] = {t[2], dx[2]}, wx[2] = {t[0], dx[0]};
    float d0 = 0.f, d1 = 0.f, d2 = 0.f;
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int c = 0; c < 2; c++) {
        d0 += (gv[1][b][c] - gv[0][b][c]) * wy[b] * wz[c];
        d1 += (gv[b][1][c] - gv[b][0][c]) * wx[b] * wz[c];
        d2 += (gv[b][c][1] - gv[b][c][0]) * wx[b] * wy[c];
      }
    gS[p] = scale * sg[0] / Ld * d0;
    gS[np + p] = scale * sg[1] / Ld * d1;
    gS[2 * np + p] = scale * sg[2] / Ld * d2;
  }
}

// out = s * sum_a D_a g_a  (the adjoint of g_a = s' D_a phi up to sign)
__global__ void k_div3(const float* __restrict__ g, int nd, float s, float* __restrict__ out) {
  const size_t ng = (size_t)nd * nd * nd;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ng; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, nd, i, j, k);
    out[c] = s * (fd6(g, 0, i, j, k, nd) + fd6(g + ng, 1, i, j, k, nd) + fd6(g + 2 * ng, 2, i, j, k, nd));
  }
}

// gradients of the six derivatives from dchi2/dsigma
__global__ void k_g6(const float* __restrict__ gsig, const float* __restrict__ d6, size_t ng, float* __restrict__ g6) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ng; c += (size_t)gridDim.x * blockDim.x) {
    const float s = gsig[c];
    const float xx = d6[c], yy = d6[ng + c], zz = d6[2 * ng + c];
    g6[c] = s * (yy + zz);
    g6[ng + c] = s * (xx + zz);
    g6[2 * ng + c] = s * (xx + yy);
    g6[3 * ng + c] = -2.f * s * d6[3 * ng + c];
    g6[4 * ng + c] = -2.f * s * d6[4 * ng + c];
    g6[5 * ng + c] = -2.f * s * d6[5 * ng + c];
  }
}

// dchi2/dS1 = dchi2/dS - (D_x gxx + D_y gxy + D_z gxz, D_y gyy + D_z gyz, D_z gzz)
__global__ void k_gS1(const float* __restrict__ gS, const float* __restrict__ g6, int nd, float inv60,
                      float* __restrict__ gS1) {
  const size_t ng = (size_t)nd * nd * nd;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ng; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, nd, i, j, k);
    const float ax = fd6(g6, 0, i, j, k, nd) + fd6(g6 + 3 * ng, 1, i, j, k, nd) + fd6(g6 + 4 * ng, 2, i, j, k, nd);
    const float ay = fd6(g6 + ng, 1, i, j, k, nd) + fd6(g6 + 5 * ng, 2, i, j, k, nd);
    const float az = fd6(g6 + 2 * ng, 2, i, j, k, nd);
    gS1[c] = gS[c] - inv60 * ax;
    gS1[ng + c] = gS[ng + c] - inv60 * ay;
    gS1[2 * ng + c] = gS[2 * ng + c] - inv60 * az;
  }
}

}  // namespace

struct DiffState {
  DevBuf buf[DB_COUNT];
  int ready = 0;
  exh_diff_params prm{};
  KnotTab T{};
  BinParams bp{};
  float L = 0.f, Lc = 0.f, Normx = 0.f, Normk = 0.f, c2 = 0.f;
  std::vector<double> bins;      // [3 Nk]: sum P, sum k, count
  std::vector<double> target, var;
};

void diff_state_release(Ctx& c) {
  if (!c.diff) return;
  for (int i = 0; i < DB_COUNT; i++) c.diff->buf[i].release();
  delete c.diff;
  c.diff = nullptr;
}

}  // namespace exh

using namespace exh;

namespace {
inline unsigned grid_for(size_t n) { return (unsigned)std::min<size_t>(exh_div_up(n, 256), (size_t)EXH_NUM_SMS * 16); }
}

extern "C" int exh_diff_forward(exh_ctx* ctx, const exh_diff_params* prm, const float* noise, const float* knot_k,
                                const float* knot_P, const float* target_P, const float* var, double* loss_out,
                                float* P_out, float* k_out, int64_t* count_out, void* stream) {
  if (!ctx || !prm || !noise || !knot_k || !knot_P || !target_P || !loss_out) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  const int nd = prm->nd;
  if (nd < 8 || nd > 1024 || (nd & 1) || prm->n_knots < 2 || prm->n_knots > MAX_KNOTS || prm->Nk < 1 ||
      prm->Nk > 4096 || !(prm->L > 0.f) || !(prm->k_max > prm->k_min)) {
    exh_set_error_msg("need even nd in [8, 1024], 2..64 knots, 1..4096 bins, L > 0, k_max > k_min", __FILE__,
                      __LINE__);
    return EXH_E_INVALID;
  }
  for (int i = 0; i < prm->n_knots; i++) {
    if (!(knot_P[i] > 0.f) || !(knot_k[i] > 0.f) || (i && !(knot_k[i] > knot_k[i - 1]))) {
      exh_set_error_msg("knots need increasing k > 0 and P > 0", __FILE__, __LINE__);
      return EXH_E_INVALID;
    }
  }
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  if (!c.diff) c.diff = new DiffState();
  DiffState& D = *c.diff;
  D.ready = 0;
  D.prm = *prm;
  const float Lc = prm->L / (float)nd;
  BoxParams b;
  EXH_TRY(setup_box(&b, nd, nd, nd, Lc, prm->Om0, prm->redshift, 1.686f, 1, 1.f, 0.f, 0.f, 1));
  D.L = b.L[0]; D.Lc = Lc; D.Normx = b.Normx; D.Normk = b.Normk;
  D.c2 = (float)(-3.0 / 7.0 * std::pow((double)b.Omz, -1.0 / 143.0));     // lpt.c:199-201
  D.T.n = prm->n_knots;
  for (int i = 0; i < D.T.n; i++) { D.T.lk[i] = logf(knot_k[i]); D.T.P[i] = knot_P[i]; }
  const int Nk = prm->Nk;
  D.target.assign(target_P, target_P + Nk);
  D.var.assign(Nk, 0.0);
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(nd, nd, nd, &p));
  const size_t ng = b.ng, nk = (size_t)nd * nd * p->nc;
  const size_t sz[DB_COUNT] = {8 * nk, 4 * nk, 8 * nk, 8 * nk, 4 * ng, 12 * ng, 24 * ng, 4 * ng, 12 * ng, 4 * ng,
                               12 * ng, 24 * ng, 12 * ng, 4 * nk, 0, 0};
  for (int i = 0; i < DB_COUNT; i++)
    if (sz[i]) EXH_TRY(D.buf[i].ensure(sz[i]));
  float2* W = D.buf[DB_W].as<float2>();
  float* A = D.buf[DB_A].as<float>();
  float2* work = D.buf[DB_WORK].as<float2>();
  float2* X = D.buf[DB_X].as<float2>();
  float* phi = D.buf[DB_PHI].as<float>();
  float* S1 = D.buf[DB_S1].as<float>();
  float* d6 = D.buf[DB_D6].as<float>();
  float* sig = D.buf[DB_SIG].as<float>();
  float* pos = D.buf[DB_POS].as<float>();
  float* grid = D.buf[DB_GRID].as<float>();
  ModeGeom g{nd, p->nc, nd / 2, (float)(2.0 * M_PI / (double)D.L)};
  const float inv60 = 1.f / (60.f * Lc);
  // field and first order
  EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{noise, nd}, work,
                          NoiseStore{W, A, work, g, D.T, (float)(1.0 / std::sqrt((double)ng))}, st));
  EXH_CUDA_TRY(fft_c2r_3d(*p, CplxLoad{work, nd, nd * p->nc}, work, RealPairStore{phi, nd, 1.f}, st));
  k_grad3<<<grid_for(ng), 256, 0, st>>>(phi, nd, -D.Normx * inv60, S1);
  count_launch(1);
  const float* phi2 = nullptr;
  if (prm->do_2lpt) {
    k_lpt2_src<<<grid_for(ng), 256, 0, st>>>(S1, nd, inv60, d6, sig);
    count_launch(1);
    EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{sig, nd}, work, PoissonStore{work, g, D.Normk}, st));
    EXH_CUDA_TRY(fft_c2r_3d(*p, CplxLoad{work, nd, nd * p->nc}, work, RealPairStore{phi, nd, 1.f}, st));
    phi2 = phi;
  }
  k_particles<<<grid_for(ng), 256, 0, st>>>(S1, phi2, nd, D.c2 * D.Normx * inv60, Lc, D.L, pos);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  // CIC and P(k)
  EXH_TRY(cic_assign(c, pos, (int64_t)ng, nd, D.L, grid, st));
  EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{grid, nd}, work, CplxStore{X, nd, nd * p->nc}, st));
  BinParams& bp = D.bp;
  bp.Nk = Nk;
  bp.kn = (float)(2 * M_PI / D.L);
  bp.kmin = prm->k_min;
  bp.dk = (prm->k_max - prm->k_min) / (float)Nk;
  bp.Lb = D.L / (float)nd;
  bp.Normk = (float)std::pow((double)(D.L / (float)(nd * nd)), 1.5);
  bp.window = 2;
  const int nblk = EXH_NUM_SMS * 2;
  const size_t hbytes = (size_t)Nk * (2 * sizeof(double) + sizeof(unsigned)) + 16;
  EXH_TRY(D.buf[DB_BINS].ensure((sizeof(double) * 2 + sizeof(unsigned)) * (size_t)nblk * Nk + 3 * sizeof(double) * Nk +
                                sizeof(float) * Nk + 256));
  double* partP = D.buf[DB_BINS].as<double>();
  double* partK = partP + (size_t)nblk * Nk;
  unsigned* partN = reinterpret_cast<unsigned*>(partK + (size_t)nblk * Nk);
  double* bins = reinterpret_cast<double*>(partN + (size_t)nblk * Nk + 2);
  bins = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(bins) + 15) & ~uintptr_t(15));
  EXH_CUDA_TRY(set_smem(k_diff_bin, hbytes));
  k_diff_bin<<<nblk, BIN_T, hbytes, st>>>(X, nk, nd, p->nc, bp, partP, partK, partN);
  k_diff_bin_reduce<<<Nk, 256, 0, st>>>(partP, partK, partN, nblk, Nk, bins);
  count_launch(2);
  EXH_CUDA_TRY(cudaGetLastError());
  D.bins.assign(3 * (size_t)Nk, 0.0);
  EXH_CUDA_TRY(cudaMemcpyAsync(D.bins.data(), bins, sizeof(double) * 3 * Nk, cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  double loss = 0.0;
  for (int i = 0; i < Nk; i++) {
    const double n = D.bins[3 * i + 2];
    const double Pb = n > 0 ? D.bins[3 * i] / n : 0.0;
    const double T = D.target[i];
    double v = var ? (double)var[i] : (n > 0 ? 2.0 * T * T / n : 0.0);
    D.var[i] = v;
    if (n > 0 && v > 0) loss += (Pb - T) * (Pb - T) / v;
    if (P_out) P_out[i] = (float)Pb;
    if (k_out) k_out[i] = n > 0 ? (float)(D.bins[3 * i + 1] / n) : 0.f;
    if (count_out) count_out[i] = (int64_t)n;
  }
  *loss_out = loss;
  D.ready = 1;
  return EXH_OK;
}

extern "C" int exh_diff_backward(exh_ctx* ctx, double grad_loss, float* grad_noise, double* grad_knots,
                                 void* stream) {
  if (!ctx || !grad_noise) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  Ctx& c = ctx->c;
  if (!c.diff || !c.diff->ready) {
    exh_set_error_msg("exh_diff_backward needs a preceding exh_diff_forward on this context", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  DiffState& D = *c.diff;
  const int nd = D.prm.nd, Nk = D.prm.Nk;
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(nd, nd, nd, &p));
  const size_t ng = (size_t)nd * nd * nd, nk = (size_t)nd * nd * p->nc;
  float2* W = D.buf[DB_W].as<float2>();
  float* A = D.buf[DB_A].as<float>();
  float2* work = D.buf[DB_WORK].as<float2>();
  float2* X = D.buf[DB_X].as<float2>();
  float* phi = D.buf[DB_PHI].as<float>();
  float* d6 = D.buf[DB_D6].as<float>();
  float* sig = D.buf[DB_SIG].as<float>();
  float* pos = D.buf[DB_POS].as<float>();
  float* ggrid = D.buf[DB_GRID].as<float>();
  float* gS = D.buf[DB_GS].as<float>();
  float* g6 = D.buf[DB_G6].as<float>();
  float* gS1 = D.buf[DB_GS1].as<float>();
  float* gA = D.buf[DB_GA].as<float>();
  ModeGeom g{nd, p->nc, nd / 2, (float)(2.0 * M_PI / (double)D.L)};
  const float inv60 = 1.f / (60.f * D.Lc);
  // dchi2/dP_b -> per-bin factor 2 g_b / N_b
  std::vector<float> gb(Nk, 0.f);
  for (int i = 0; i < Nk; i++) {
    const double n = D.bins[3 * i + 2];
    if (n > 0 && D.var[i] > 0) {
      const double Pb = D.bins[3 * i] / n;
      gb[i] = (float)(grad_loss * 2.0 * (Pb - D.target[i]) / D.var[i] * 2.0 / n);
    }
  }
  EXH_TRY(D.buf[DB_KNOTS].ensure(sizeof(float) * Nk + sizeof(double) * ((size_t)EXH_NUM_SMS * 2 * MAX_KNOTS + MAX_KNOTS) +
                                 64));
  float* gbin = D.buf[DB_KNOTS].as<float>();
  double* kpart = reinterpret_cast<double*>(reinterpret_cast<char*>(gbin) + ((sizeof(float) * Nk + 15) & ~size_t(15)));
  double* kout = kpart + (size_t)EXH_NUM_SMS * 2 * MAX_KNOTS;
  if (sizeof(float) * Nk <= UPLOAD_SMALL_MAX) {
    EXH_TRY(upload_small(gbin, gb.data(), sizeof(float) * Nk, st));
  } else {
    EXH_CUDA_TRY(cudaMemcpyAsync(gbin, gb.data(), sizeof(float) * Nk, cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));      // gb dies at return
  }
  // P(k) and r2c adjoint: dchi2/dgrid
  EXH_CUDA_TRY(fft_c2r_3d(*p, BinGradLoad{X, gbin, g, D.bp}, work, RealPairStore{ggrid, nd, 1.f}, st));
  // CIC adjoint: delta = rho * ng / np - 1 with np = ng
  k_cic_adjoint<<<grid_for(ng), 256, 0, st>>>(pos, ng, nd, D.L, D.L / (float)nd, 1.f, ggrid, gS);
  count_launch(1);
  const float sx = D.Normx * inv60;        // S1 = -sx R phi1;  S2 = c2 sx R phi2
  if (D.prm.do_2lpt) {
    // phi2: dchi2/dphi2 = -c2 sx sum_a R_a gS_a
    k_div3<<<grid_for(ng), 256, 0, st>>>(gS, nd, -D.c2 * sx, phi);
    count_launch(1);
    // sigma: c2r(r2c(.) Normk / (-k^2)); the half-plane factors of the two adjoints cancel
    EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{phi, nd}, work, PoissonStore{work, g, D.Normk}, st));
    EXH_CUDA_TRY(fft_c2r_3d(*p, CplxLoad{work, nd, nd * p->nc}, work, RealPairStore{sig, nd, 1.f}, st));
    k_g6<<<grid_for(ng), 256, 0, st>>>(sig, d6, ng, g6);
    k_gS1<<<grid_for(ng), 256, 0, st>>>(gS, g6, nd, inv60, gS1);
    count_launch(2);
  } else {
    EXH_CUDA_TRY(cudaMemcpyAsync(gS1, gS, sizeof(float) * 3 * ng, cudaMemcpyDeviceToDevice, st));
  }
  // phi1: dchi2/dphi1 = sx sum_a R_a gS1_a
  k_div3<<<grid_for(ng), 256, 0, st>>>(gS1, nd, sx, phi);
  count_launch(1);
  EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{phi, nd}, work, NoiseGradStore{W, A, work, gA, g}, st));
  EXH_CUDA_TRY(fft_c2r_3d(*p, CplxLoad{work, nd, nd * p->nc}, work, RealPairStore{grad_noise, nd, 1.f}, st));
  if (grad_knots) {
    const int nblk = EXH_NUM_SMS * 2;
    k_knot_grad<<<nblk, BIN_T, 0, st>>>(gA, A, nk, g, D.T, kpart);
    k_knot_reduce<<<D.T.n, 256, 0, st>>>(kpart, nblk, D.T.n, kout);
    count_launch(2);
    EXH_CUDA_TRY(cudaGetLastError());
    EXH_CUDA_TRY(cudaMemcpyAsync(grad_knots, kout, sizeof(double) * D.T.n, cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
  }
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}
