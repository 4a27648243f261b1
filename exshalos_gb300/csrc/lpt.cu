// Lagrangian perturbation theory (src/exshalos/lpt.c:4-255).
//
// 1LPT: phi_k = -delta_k / k^2 is generated inside the first pass of the
//       inverse FFT from the same Philox modes as the field (nothing is read
//       from k space); S1 = -D6(phi) Normx / (60 Lc) with the sixth-order
//       central difference of lpt.c:64-68.
// 2LPT: the source sum_{i<j} (d_i S_i d_j S_j - (d_j S_i)^2) (lpt.c:116-134)
//       is transformed forward, multiplied by Normk / (-k^2) and transformed
//       back inside one fused x pass; S2 = D6(phi2) Normx / (60 Lc) *
//       (-3/7) Omega_m(z)^(-1/143) (lpt.c:190-198).
// Halo sums: one warp per halo walks its member shells in a fixed order and
// reduces in FP64 (lpt.c:70-80, 200-210, 245-255).
#include <cmath>

#include "ctx.cuh"
#include "fft4.cuh"
#include "fp32sum.cuh"
#include "field.cuh"
#include "halos.cuh"
#include "lpt.cuh"
#include "scan.cuh"

namespace exh {

struct KGrid {
  int n0, n1, n2;
  float kl0, kl1, kl2;
  float k_smooth;
  // float wave numbers as the reference forms them (lpt.c:13-29)
  __device__ __forceinline__ float k2(int i, int j, int k, float& kmod) const {
    const float kx = (float)((2 * i < n0) ? i : i - n0) * kl0;
    const float ky = (float)((2 * j < n1) ? j : j - n1) * kl1;
    float kz = (float)k * kl2;
    if (k == n2 / 2) kz = -(float)(n2 / 2) * kl2;
    const float s = kx * kx + ky * ky + kz * kz;
    kmod = sqrtf(s);
    return s;
  }
};

// x-pass source of the first-order potential
struct Lpt1Gen {
  static constexpr int io_bytes = 0;
  FieldModes m;
  KGrid g;
  __device__ __forceinline__ float2 operator()(int, int e, int inner) const {
    const int j = inner / m.nc, k = inner % m.nc;
    float kmod;
    const float s = g.k2(e, j, k, kmod);
    if (s == 0.f || kmod > g.k_smooth) return make_float2(0.f, 0.f);
    const float2 v = m.mode(e, j, k);
    const float f = -(kmod * kmod);
    return make_float2(v.x / f, v.y / f);
  }
};

// ---------------------------------------------------------------- stencils
// Sixth-order central differences (1, -9, 45, 0, -45, 9, -1) / 60 of
// lpt.c:64-68 on shared-memory bricks with a 3-cell periodic halo; the
// differences of opposite neighbours are formed first, which keeps float
// accuracy on smooth fields.
constexpr int BZ = 32, BY = 8;
constexpr int GX = 16;            // bricks of 16 x 8 x 32 cells for gradients
constexpr int SX = 8;             // bricks of 8 x 8 x 32 cells for the 2LPT source
constexpr int H = 3;

__device__ __forceinline__ float d6f(float p1, float p2, float p3, float m1, float m2, float m3) {
  return (p3 - m3) - 9.f * (p2 - m2) + 45.f * (p1 - m1);
}

// load an EX x EY x EZ tile whose origin is (x0 - hx, y0 - hy, z0 - hz);
// the extents are compile-time, so the index split costs no division
template <int EX, int EY, int EZ>
__device__ __forceinline__ void load_tile(const float* __restrict__ f, float* t, int x0, int y0, int z0, int hx,
                                          int hy, int hz, int n0, int n1, int n2) {
  constexpr int tot = EX * EY * EZ;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  const bool small = (size_t)n0 * n1 * n2 <= 0xffffffffull;     // 32-bit cell indexes
  for (int q = tid; q < tot; q += nt) {
    const int dz = q % EZ, r = q / EZ, dy = r % EY, dx = r / EY;
    const int gx = exh_wrap(x0 - hx, dx, n0), gy = exh_wrap(y0 - hy, dy, n1), gz = exh_wrap(z0 - hz, dz, n2);
    t[q] = small ? f[((uint32_t)gx * (uint32_t)n1 + (uint32_t)gy) * (uint32_t)n2 + (uint32_t)gz]
                 : f[((size_t)gx * n1 + gy) * n2 + gz];
  }
}

// S[a] (=|+=) fac * D6_a(phi); V[a] (=|+=) fv * fac * D6_a(phi) when V
template <bool ADD>
__global__ void __launch_bounds__(256)
k_brick_grad(const float* __restrict__ phi, int n0, int n1, int n2, float fac, float fv, float* __restrict__ S,
             float* __restrict__ V) {
  extern __shared__ float tile[];
  constexpr int EY = BY + 2 * H, EZ = BZ + 2 * H;
  const int z0 = blockIdx.x * BZ, y0 = blockIdx.y * BY, x0 = blockIdx.z * GX;
  load_tile<GX + 2 * H, EY, EZ>(phi, tile, x0, y0, z0, H, H, H, n0, n1, n2);
  __syncthreads();
  const int tz = threadIdx.x, ty = threadIdx.y;
  const int gz = z0 + tz, gy = y0 + ty;
  if (gz >= n2 || gy >= n1) return;
  const size_t ng = (size_t)n0 * n1 * n2;
  for (int xx = 0; xx < GX && x0 + xx < n0; xx++) {
    const int cx = xx + H, cy = ty + H, cz = tz + H;
#define T(a, b, c) tile[((a) * EY + (b)) * EZ + (c)]
    const float g[3] = {
        d6f(T(cx + 1, cy, cz), T(cx + 2, cy, cz), T(cx + 3, cy, cz), T(cx - 1, cy, cz), T(cx - 2, cy, cz), T(cx - 3, cy, cz)),
        d6f(T(cx, cy + 1, cz), T(cx, cy + 2, cz), T(cx, cy + 3, cz), T(cx, cy - 1, cz), T(cx, cy - 2, cz), T(cx, cy - 3, cz)),
        d6f(T(cx, cy, cz + 1), T(cx, cy, cz + 2), T(cx, cy, cz + 3), T(cx, cy, cz - 1), T(cx, cy, cz - 2), T(cx, cy, cz - 3))};
#undef T
    const size_t c = ((size_t)(x0 + xx) * n1 + gy) * n2 + gz;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float s = g[a] * fac;
      if (ADD) S[a * ng + c] += s; else S[a * ng + c] = s;
      if (V) { if (ADD) V[a * ng + c] += fv * s; else V[a * ng + c] = fv * s; }
    }
  }
}

// second-order source (lpt.c:116-134) from the first-order displacement
__global__ void __launch_bounds__(256)
k_brick_source(const float* __restrict__ S, int n0, int n1, int n2, float inv60lc, float* __restrict__ src) {
  extern __shared__ float sm[];
  constexpr int EY = BY + 2 * H, EZ = BZ + 2 * H;
  float* tx = sm;                                  // Sx: halo in x, y, z
  float* ty_ = tx + (SX + 2 * H) * EY * EZ;         // Sy: halo in y, z
  float* tz_ = ty_ + SX * EY * EZ;                  // Sz: halo in z
  const size_t ng = (size_t)n0 * n1 * n2;
  const int z0 = blockIdx.x * BZ, y0 = blockIdx.y * BY, x0 = blockIdx.z * SX;
  load_tile<SX + 2 * H, EY, EZ>(S, tx, x0, y0, z0, H, H, H, n0, n1, n2);
  load_tile<SX, EY, EZ>(S + ng, ty_, x0, y0, z0, 0, H, H, n0, n1, n2);
  load_tile<SX, BY, EZ>(S + 2 * ng, tz_, x0, y0, z0, 0, 0, H, n0, n1, n2);
  __syncthreads();
  const int tzz = threadIdx.x, tyy = threadIdx.y;
  const int gz = z0 + tzz, gy = y0 + tyy;
  if (gz >= n2 || gy >= n1) return;
  for (int xx = 0; xx < SX && x0 + xx < n0; xx++) {
    const int cz = tzz + H, cy = tyy + H;
#define AX(a, b, c) tx[((a) * EY + (b)) * EZ + (c)]
#define AY(a, b, c) ty_[((a) * EY + (b)) * EZ + (c)]
#define AZ(a, b, c) tz_[((a) * BY + (b)) * EZ + (c)]
    const int cx = xx + H;
    const float pxx = inv60lc * d6f(AX(cx + 1, cy, cz), AX(cx + 2, cy, cz), AX(cx + 3, cy, cz), AX(cx - 1, cy, cz), AX(cx - 2, cy, cz), AX(cx - 3, cy, cz));
    const float pxy = inv60lc * d6f(AX(cx, cy + 1, cz), AX(cx, cy + 2, cz), AX(cx, cy + 3, cz), AX(cx, cy - 1, cz), AX(cx, cy - 2, cz), AX(cx, cy - 3, cz));
    const float pxz = inv60lc * d6f(AX(cx, cy, cz + 1), AX(cx, cy, cz + 2), AX(cx, cy, cz + 3), AX(cx, cy, cz - 1), AX(cx, cy, cz - 2), AX(cx, cy, cz - 3));
    const float pyy = inv60lc * d6f(AY(xx, cy + 1, cz), AY(xx, cy + 2, cz), AY(xx, cy + 3, cz), AY(xx, cy - 1, cz), AY(xx, cy - 2, cz), AY(xx, cy - 3, cz));
    const float pyz = inv60lc * d6f(AY(xx, cy, cz + 1), AY(xx, cy, cz + 2), AY(xx, cy, cz + 3), AY(xx, cy, cz - 1), AY(xx, cy, cz - 2), AY(xx, cy, cz - 3));
    const float pzz = inv60lc * d6f(AZ(xx, tyy, cz + 1), AZ(xx, tyy, cz + 2), AZ(xx, tyy, cz + 3), AZ(xx, tyy, cz - 1), AZ(xx, tyy, cz - 2), AZ(xx, tyy, cz - 3));
#undef AX
#undef AY
#undef AZ
    const float diag = pxx * pyy + pxx * pzz + pyy * pzz;
    src[((size_t)(x0 + xx) * n1 + gy) * n2 + gz] = source_combine(diag, pxy, pxz, pyz);
  }
}

// Poisson factor of mode (e, col) of the x pass: Normk / (-k^2), zero at
// k = 0 and above k_smooth (lpt.c:140-150)
__device__ __forceinline__ float2 poisson_mode(float2 v, const KGrid& g, int e, int col, int nc, float normk) {
  float kmod;
  const float s = g.k2(e, col / nc, col % nc, kmod);
  if (s == 0.f || kmod > g.k_smooth) return make_float2(0.f, 0.f);
  const float f = -(kmod * kmod);
  return make_float2(v.x / f * normk, v.y / f * normk);
}

// x pass of the 2LPT Poisson solve as register four-step FFTs (fft4.cuh):
// forward, x Normk/(-k^2), inverse, on a tile of W columns; the modes go
// back to shared memory in natural order between the two transforms.
template <int N1, int N2>
__global__ void __launch_bounds__(FS_THREADS, 2)
k_fft4_x_poisson(float2* __restrict__ work, const float2* __restrict__ tw, int inner, KGrid g, float normk) {
  using S = FsShape<N1, N2>;
  constexpr int W = S::W, n = S::n;
  __shared__ float2 sm[n * W];
  const int i0 = blockIdx.x * W;
  const int nb = min(W, inner - i0);
  const int c = threadIdx.x % W, jj = threadIdx.x / W;
  const int nc = g.n2 / 2 + 1;
  const bool live = c < nb;
  float2 v[N1];
  float2 u[N2];
  if (jj < N2) {
#pragma unroll
    for (int j1 = 0; j1 < N1; j1++)
      v[j1] = live ? work[(size_t)(jj + N2 * j1) * inner + i0 + c] : make_float2(0.f, 0.f);
    RDft<N1>::run(v, -1.f, [tw](int m) { return __ldg(&tw[m * N2]); });
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) {
      float2 x = v[k1];
      if (k1 != 0 && jj != 0) x = cmul(x, tw_get(tw, jj * k1, -1.f));
      sm[(k1 * N2 + jj) * W + c] = x;
    }
  }
  __syncthreads();
  if (jj < N1) {
#pragma unroll
    for (int j2 = 0; j2 < N2; j2++) u[j2] = sm[(jj * N2 + j2) * W + c];
    RDft<N2>::run(u, -1.f, [tw](int m) { return __ldg(&tw[m * N1]); });
#pragma unroll
    for (int k2 = 0; k2 < N2; k2++)
      u[k2] = live ? poisson_mode(u[k2], g, jj + N1 * k2, i0 + c, nc, normk) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  if (jj < N1) {
#pragma unroll
    for (int k2 = 0; k2 < N2; k2++) sm[(jj + N1 * k2) * W + c] = u[k2];
  }
  __syncthreads();
  if (jj < N2) {
#pragma unroll
    for (int j1 = 0; j1 < N1; j1++) v[j1] = sm[(jj + N2 * j1) * W + c];
  }
  __syncthreads();
  if (jj < N2) {
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
#pragma unroll
    for (int j2 = 0; j2 < N2; j2++) u[j2] = sm[(jj * N2 + j2) * W + c];
    RDft<N2>::run(u, 1.f, [tw](int m) { return __ldg(&tw[m * N1]); });
    if (live) {
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) work[(size_t)(jj + N1 * k2) * inner + i0 + c] = u[k2];
    }
  }
}

// The same for length 512 on the three radix-8 stages of k_fft8_strided512.
__global__ void __launch_bounds__(F512_T, 2)
k_fft8_x_poisson512(float2* __restrict__ work, const float2* __restrict__ tw, int inner, KGrid g, float normk) {
  __shared__ float2 sm[(512 + 64) * F512_W];
  const int i0 = blockIdx.x * F512_W;
  const int nb = min(F512_W, inner - i0);
  const int c = threadIdx.x % F512_W, q = threadIdx.x / F512_W;
  const int nc = g.n2 / 2 + 1;
  const bool live = c < nb;
  const int k1 = q >> 3, k2a = q & 7;
  float2 v[8];
  f512_run([&](int j) { return live ? work[(size_t)j * inner + i0 + c] : make_float2(0.f, 0.f); }, sm, tw, -1.f,
           c, q, v);
#pragma unroll
  for (int k2b = 0; k2b < 8; k2b++)
    v[k2b] = live ? poisson_mode(v[k2b], g, k1 + 8 * k2a + 64 * k2b, i0 + c, nc, normk) : make_float2(0.f, 0.f);
  __syncthreads();
#pragma unroll
  for (int k2b = 0; k2b < 8; k2b++) sm[f512_at(k1 + 8 * k2a + 64 * k2b, c)] = v[k2b];
  __syncthreads();
#pragma unroll
  for (int j1 = 0; j1 < 8; j1++) v[j1] = sm[f512_at(q + 64 * j1, c)];
  __syncthreads();
  f512_core(v, sm, tw, 1.f, c, q);
  if (live) {
#pragma unroll
    for (int k2b = 0; k2b < 8; k2b++) work[(size_t)(k1 + 8 * k2a + 64 * k2b) * inner + i0 + c] = v[k2b];
  }
}

// x pass of the 2LPT Poisson solve: forward, x Normk/(-k^2), inverse
// (shared-memory Stockham, for lengths without a register split)
__global__ void __launch_bounds__(FFT_THREADS)
k_fft_x_poisson(float2* __restrict__ work, RadixPlan pl, const float2* __restrict__ tw, int inner, KGrid g,
                float normk) {
  extern __shared__ float2 smem[];
  const int n = pl.n;
  float2* b0 = smem;
  float2* b1 = smem + n * FFT_W;
  const int i0 = blockIdx.x * FFT_W;
  const int nb = min(FFT_W, inner - i0);
  const int nc = g.n2 / 2 + 1;
  for (int t = threadIdx.x; t < n * FFT_W; t += blockDim.x) {
    const int e = t / FFT_W, b = t % FFT_W;
    b0[e * FFT_W + b] = (b < nb) ? work[(size_t)e * inner + i0 + b] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* res = stockham_run(b0, b1, pl, FFT_W, FFT_W, tw, -1.f);
  for (int t = threadIdx.x; t < n * FFT_W; t += blockDim.x) {
    const int e = t / FFT_W, b = t % FFT_W;
    const int col = i0 + b;
    float2 v = res[e * FFT_W + b];
    if (b < nb) v = poisson_mode(v, g, e, col, nc, normk);
    res[e * FFT_W + b] = v;
  }
  __syncthreads();
  float2* other = (res == b0) ? b1 : b0;
  float2* out = stockham_run(res, other, pl, FFT_W, FFT_W, tw, 1.f);
  for (int t = threadIdx.x; t < n * FFT_W; t += blockDim.x) {
    const int e = t / FFT_W, b = t % FFT_W;
    if (b < nb) work[(size_t)e * inner + i0 + b] = out[e * FFT_W + b];
  }
}

// ---------------------------------------------------------------- halos
// Displacement and velocity sums over the member cells of each halo
// (lpt.c:70-80, 200-210) and the final positions (lpt.c:245-255): halos of
// at most HS_LANE_MAX cells by one thread each, the others by one warp each.
// The order of every sum is fixed, so the result is deterministic.
// Halo position (and velocity) from the member sums: cysumf(x Lc + Lc / 2,
// disp / count, L) per axis, exshalos_h.c:13-19
__device__ __forceinline__ void halo_write(int64_t h, int cnt, const int xc[3], const double s[3], const double v[3],
                                           const HaloOut& o) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float disp = (float)s[a];
    const float xq = (float)((double)((float)xc[a] * o.Lc) + (double)o.Lc / 2.0);
    float p = xq + disp / (float)cnt;
    if (p >= o.L[a]) p -= o.L[a];
    if (p < 0.f) p += o.L[a];
    o.posh[3 * h + a] = p;
    if (o.velh) o.velh[3 * h + a] = (float)(v[a] / (double)cnt);
  }
}

__device__ __forceinline__ size_t hs_cell(const int* __restrict__ off_all, int q, int xa, int ya, int za, int n0,
                                          int n1, int n2) {
  const int pk = off_all[q];
  const int i = exh_wrap(xa, (pk & 0xff) - 128, n0), j = exh_wrap(ya, ((pk >> 8) & 0xff) - 128, n1),
            k = exh_wrap(za, ((pk >> 16) & 0xff) - 128, n2);
  return ((size_t)i * n1 + j) * n2 + k;
}

__device__ __forceinline__ void hs_centre(const int* __restrict__ hpeak, const int* __restrict__ gfin,
                                          const unsigned* __restrict__ pid, int64_t np,
                                          const int* __restrict__ start_all, int64_t h, int n1, int n2, int xc[3],
                                          int& cnt) {
  const int r = hpeak[h];
  const unsigned cell0 = pid[np - 1 - r];
  xc[2] = (int)(cell0 % n2);
  const unsigned rr = cell0 / n2;
  xc[1] = (int)(rr % n1);
  xc[0] = (int)(rr / n1);
  cnt = start_all[gfin[r]];
}

// Member sums of the halos (Compute_Posh, lpt.c:229-255): each member's
// term in a compensated FP32 sum (FSum), FP64 once per halo.  Most halos are
// one cell (at box_256, 83 %); a warp whose lanes mixed them with large
// halos ran as long as its largest, so this pass sums the halos of at most
// HS_LANE_MAX members, one thread each, and hands the others (one atomic per
// block) to k_halo_sum_warp.
constexpr int HS_LANE_MAX = 7;
__global__ void __launch_bounds__(256)
k_halo_sum(const int* __restrict__ hpeak, const int* __restrict__ gfin, const unsigned* __restrict__ pid, int64_t np,
           int64_t nh, const int* __restrict__ off_all, const int* __restrict__ start_all, const float* __restrict__ S,
           const float* __restrict__ V, int n0, int n1, int n2, HaloOut o, int* __restrict__ big,
           int* __restrict__ nbig) {
  __shared__ int ws[32];
  __shared__ int base;
  const int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = h < nh;
  const size_t ng = (size_t)n0 * n1 * n2;
  int xc[3] = {0, 0, 0}, cnt = 0;
  if (valid) hs_centre(hpeak, gfin, pid, np, start_all, h, n1, n2, xc, cnt);
  const bool mine = valid && cnt <= HS_LANE_MAX;
  if (mine) {
    FSum fs[3], fv[3];
#pragma unroll
    for (int q = 0; q < HS_LANE_MAX; q++) {
      if (q >= cnt) break;
      const size_t c = hs_cell(off_all, q, xc[0], xc[1], xc[2], n0, n1, n2);
#pragma unroll
      for (int a = 0; a < 3; a++) {
        fs[a].add(S[a * ng + c]);
        if (V) fv[a].add(V[a * ng + c]);
      }
    }
    double s[3], v[3];
#pragma unroll
    for (int a = 0; a < 3; a++) { s[a] = fs[a].value(); v[a] = fv[a].value(); }
    halo_write(h, cnt, xc, s, v, o);
  }
  const int hand = (valid && !mine) ? 1 : 0;
  int tot;
  const int ex = block_exclusive_scan<int>(hand, ws, tot);
  if (threadIdx.x == 0 && tot) base = atomicAdd(nbig, tot);
  __syncthreads();
  if (hand) big[base + ex] = (int)h;
}

// the larger halos, one warp each (persistent): lane-strided compensated
// sums, the 32 partial values added in FP64 by a butterfly
__global__ void __launch_bounds__(256)
k_halo_sum_warp(const int* __restrict__ hpeak, const int* __restrict__ gfin, const unsigned* __restrict__ pid,
                int64_t np, const int* __restrict__ off_all, const int* __restrict__ start_all,
                const float* __restrict__ S, const float* __restrict__ V, int n0, int n1, int n2, HaloOut o,
                const int* __restrict__ big, const int* __restrict__ nbig) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  const int n = *nbig;
  const size_t ng = (size_t)n0 * n1 * n2;
  for (int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); w < n; w += nwarps) {
    const int64_t h = big[w];
    int xc[3], cnt;
    hs_centre(hpeak, gfin, pid, np, start_all, h, n1, n2, xc, cnt);
    FSum fs[3], fv[3];
#pragma unroll 4
    for (int q = lane; q < cnt; q += 32) {
      const size_t c = hs_cell(off_all, q, xc[0], xc[1], xc[2], n0, n1, n2);
#pragma unroll
      for (int a = 0; a < 3; a++) {
        fs[a].add(S[a * ng + c]);
        if (V) fv[a].add(V[a * ng + c]);
      }
    }
    double ts[3], tv[3];
#pragma unroll
    for (int a = 0; a < 3; a++) { ts[a] = fs[a].value(); tv[a] = fv[a].value(); }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int ww = 16; ww > 0; ww >>= 1) {
        ts[a] += __shfl_xor_sync(0xffffffffu, ts[a], ww);
        tv[a] += __shfl_xor_sync(0xffffffffu, tv[a], ww);
      }
    if (lane == 0) halo_write(h, cnt, xc, ts, tv, o);
  }
}

// particle positions q + S and velocities (lpt.c:82-92, 212-222, 229-242),
// interleaved [ng][3]
// The lattice coordinate (x + 1/2) Lc of every index of the three axes is
// formed once per block (the reference's float product plus a double half
// cell) into shared memory (n0 + n1 + n2 floats).
__global__ void k_particles(const float* __restrict__ S, const float* __restrict__ V, int n0, int n1, int n2,
                            HaloOut o, float* __restrict__ pos, float* __restrict__ vel) {
  extern __shared__ float xq_s[];
  for (int t = threadIdx.x; t < n0 + n1 + n2; t += blockDim.x) {
    const int x = t < n0 ? t : (t < n0 + n1 ? t - n0 : t - n0 - n1);
    xq_s[t] = (float)((double)((float)x * o.Lc) + (double)o.Lc / 2.0);
  }
  __syncthreads();
  const int base[3] = {0, n0, n0 + n1};
  const size_t ng = (size_t)n0 * n1 * n2;
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; c < ng; c += stride) {
    int i, j, k;
    cell_ijk(c, ng, n1, n2, &i, &j, &k);
    const int xc[3] = {i, j, k};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float xq = xq_s[base[a] + xc[a]];
      float p = xq + S[a * ng + c];
      if (p >= o.L[a]) p -= o.L[a];
      if (p < 0.f) p += o.L[a];
      pos[3 * c + a] = p;
      if (vel) vel[3 * c + a] = V[a * ng + c];
    }
  }
}

float lpt2_factor(const BoxParams& b) {
  // D6(phi2) Normx / (60 Lc) then (-3/7) Omega_m(z)^(-1/143), lpt.c:190-198
  return (float)(b.Normx / (60.0 * b.Lc) * (-3.0 / 7.0 * std::pow((double)b.Omz, -1.0 / 143)));
}

HaloOut make_halo_out(const BoxParams& b, float* posh, float* velh) {
  HaloOut o;
  o.posh = posh;
  o.velh = velh;
  o.Lc = b.Lc;
  for (int a = 0; a < 3; a++) o.L[a] = b.L[a];
  o.f1 = std::pow((double)b.Omz, 0.5454) * b.Hz / (1.0 + b.redshift);
  o.f2 = 2.0 * std::pow((double)b.Omz, 6.0 / 11.0) * b.Hz / (1.0 + b.redshift);
  return o;
}

static cudaError_t launch_grad(const BoxParams& b, const float* phi, float fac, float fv, float* S, float* V, bool add,
                               cudaStream_t st) {
  const dim3 grid(exh_div_up(b.nd[2], BZ), exh_div_up(b.nd[1], BY), exh_div_up(b.nd[0], GX));
  const size_t sm = sizeof(float) * (GX + 2 * H) * (BY + 2 * H) * (BZ + 2 * H);
  auto kern = add ? k_brick_grad<true> : k_brick_grad<false>;
  cudaError_t e = set_smem(kern, sm);
  if (e != cudaSuccess) return e;
  KTimer kt(KC_LPT_STENCIL, st, (4.0 + (add ? 24.0 : 12.0) * (V ? 2 : 1)) * b.ng);
  kern<<<grid, dim3(BZ, BY), sm, st>>>(phi, b.nd[0], b.nd[1], b.nd[2], fac, fv, S, V);
  count_launch(1);
  return cudaGetLastError();
}

// x pass of r2c(delta) for a given field (Compute_Denk, density_grid.c:220-235,
// then lpt.c:11-45): phi1_k = Normk delta_k / (-k^2), 0 at k = 0 and k > k_smooth
struct Lpt1FromGrid {
  static constexpr int io_bytes = 8;
  float2* __restrict__ out;
  KGrid g;
  int nc;
  float Normk;
  __device__ __forceinline__ void operator()(int, int e, int inner, float2 v) const {
    const int j = inner / nc, k = inner % nc;
    float kmod;
    const float s = g.k2(e, j, k, kmod);
    float2 r = make_float2(0.f, 0.f);
    if (s != 0.f && kmod <= g.k_smooth) {
      const float f = -(kmod * kmod);
      r = make_float2(Normk * v.x / f, Normk * v.y / f);
    }
    out[(size_t)e * ((size_t)g.n1 * nc) + inner] = r;
  }
};

static int lpt_from_phi1(Ctx& c, const BoxParams& b, float k_smooth, bool do2, float* S, float* V, float* phi1,
                         float* phi2, cudaStream_t st);

int lpt_run(Ctx& c, const BoxParams& b, const FieldModes& modes, float k_smooth, bool do2, float* S, float* V,
            float* phi1, float* phi2, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
  const size_t nk = (size_t)b.nd[0] * b.nd[1] * p->nc;
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  float2* work = c.buf[B_WORK].as<float2>();
  KGrid g{b.nd[0], b.nd[1], b.nd[2], b.kl[0], b.kl[1], b.kl[2], k_smooth};
  EXH_CUDA_TRY(fft_c2r_3d(*p, Lpt1Gen{modes, g}, work, RealPairStore{phi1, b.nd[2], 1.f}, st));
  return lpt_from_phi1(c, b, k_smooth, do2, S, V, phi1, phi2, st);
}

int lpt_run_grid(Ctx& c, const BoxParams& b, const float* delta, float k_smooth, bool do2, float* S, float* V,
                 float* phi1, float* phi2, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
  const size_t nk = (size_t)b.nd[0] * b.nd[1] * p->nc;
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  float2* work = c.buf[B_WORK].as<float2>();
  KGrid g{b.nd[0], b.nd[1], b.nd[2], b.kl[0], b.kl[1], b.kl[2], k_smooth};
  EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{delta, b.nd[2]}, work, Lpt1FromGrid{work, g, p->nc, b.Normk}, st));
  EXH_CUDA_TRY(fft_c2r_3d(*p, CplxLoad{work, b.nd[0], b.nd[1] * p->nc}, work, RealPairStore{phi1, b.nd[2], 1.f}, st));
  return lpt_from_phi1(c, b, k_smooth, do2, S, V, phi1, phi2, st);
}

static int lpt_from_phi1(Ctx& c, const BoxParams& b, float k_smooth, bool do2, float* S, float* V, float* phi1,
                         float* phi2, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
  float2* work = c.buf[B_WORK].as<float2>();
  const HaloOut o = make_halo_out(b, nullptr, nullptr);
  KGrid g{b.nd[0], b.nd[1], b.nd[2], b.kl[0], b.kl[1], b.kl[2], k_smooth};
  // S1 = -D6(phi1) Normx / (60 Lc)  (lpt.c:64-68)
  EXH_CUDA_TRY(launch_grad(b, phi1, (float)(-b.Normx / (60.0 * b.Lc)), (float)o.f1, S, V, false, st));
  if (!do2) return EXH_OK;
  float* src = phi2;   // the source is transformed, then phi2 overwrites it
  {
    const dim3 grid(exh_div_up(b.nd[2], BZ), exh_div_up(b.nd[1], BY), exh_div_up(b.nd[0], SX));
    const size_t sm = sizeof(float) * (BY + 2 * H) * (BZ + 2 * H) * ((SX + 2 * H) + SX) +
                      sizeof(float) * SX * BY * (BZ + 2 * H);
    EXH_CUDA_TRY(set_smem(k_brick_source, sm));
    KTimer kt(KC_LPT_STENCIL, st, 16.0 * b.ng);
    k_brick_source<<<grid, dim3(BZ, BY), sm, st>>>(S, b.nd[0], b.nd[1], b.nd[2], (float)(1.0 / (60.0 * b.Lc)), src);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  const size_t rows = (size_t)b.nd[0] * b.nd[1];
  EXH_CUDA_TRY(launch_r2c_rows(RealPairLoad{src, b.nd[2]}, HalfStore{work, p->nc}, *p, rows, st));
  EXH_CUDA_TRY(launch_strided(CplxLoad{work, b.nd[1], p->nc}, CplxStore{work, b.nd[1], p->nc}, p->py, p->twy, -1.f,
                              b.nd[0], p->nc, st));
  const int inner = b.nd[1] * p->nc;
  {
    KTimer kt(KC_FFT_STRIDED, st, 16.0 * b.nd[0] * inner);
    if (b.nd[0] == 512) {
      k_fft8_x_poisson512<<<exh_div_up(inner, F512_W), F512_T, 0, st>>>(work, p->twx, inner, g, b.Normk);
    } else {
      switch (fs_split(b.nd[0])) {
#define X(A_, B_)                                                                                       \
  case A_ * 1000 + B_:                                                                                  \
    k_fft4_x_poisson<A_, B_><<<exh_div_up(inner, FsShape<A_, B_>::W), FS_THREADS, 0, st>>>(work, p->twx, inner, g, \
                                                                                       b.Normk);         \
    break;
        EXH_FS_STRIDED_CASES(X)
#undef X
        default: {
          const size_t sm = smem_strided(b.nd[0]);
          EXH_CUDA_TRY(set_smem(k_fft_x_poisson, sm));
          k_fft_x_poisson<<<exh_div_up(inner, FFT_W), FFT_THREADS, sm, st>>>(work, p->px, p->twx, inner, g, b.Normk);
        }
      }
    }
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  EXH_CUDA_TRY(launch_strided(CplxLoad{work, b.nd[1], p->nc}, CplxStore{work, b.nd[1], p->nc}, p->py, p->twy, 1.f,
                              b.nd[0], p->nc, st));
  EXH_CUDA_TRY(launch_c2r_rows(HalfLoad{work, p->nc}, RealPairStore{phi2, b.nd[2], 1.f}, *p, rows, st));
  // S += S2, V += f2 S2 with S2 = D6(phi2) Normx / (60 Lc) (-3/7) Omega^(-1/143)
  EXH_CUDA_TRY(launch_grad(b, phi2, lpt2_factor(b), (float)o.f2, S, V, true, st));
  return EXH_OK;
}

int halo_displacements(Ctx& c, const BoxParams& b, const HaloDev& h, const ShellTable& t, const float* S,
                       const float* V, const HaloOut& o, cudaStream_t st) {
  if (h.nh == 0) return EXH_OK;
  EXH_TRY(c.buf[B_HSUM].ensure(sizeof(int) * ((size_t)h.nh + 64)));
  int* nbig = c.buf[B_HSUM].as<int>();
  int* big = nbig + 32;
  EXH_CUDA_TRY(cudaMemsetAsync(nbig, 0, sizeof(int), st));
  KTimer kt(KC_HALO_DISP, st, 0.0);
  k_halo_sum<<<exh_div_up(h.nh, 256), 256, 0, st>>>(h.hpeak, h.gfin, h.id, h.np, h.nh, t.off_all, t.start_all, S, V,
                                                    b.nd[0], b.nd[1], b.nd[2], o, big, nbig);
  k_halo_sum_warp<<<EXH_NUM_SMS * 8, 256, 0, st>>>(h.hpeak, h.gfin, h.id, h.np, t.off_all, t.start_all, S, V,
                                                  b.nd[0], b.nd[1], b.nd[2], o, big, nbig);
  count_launch(2);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

// [ng][3] -> planes [3][ng]
__global__ void k_aos_to_planes(const float* __restrict__ in, size_t ng, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < 3 * ng; i += (size_t)gridDim.x * blockDim.x) {
    const size_t c = i / 3;
    const int a = (int)(i % 3);
    out[a * ng + c] = in[i];
  }
}

int aos_to_planes(const float* in, size_t ng, float* out, cudaStream_t st) {
  k_aos_to_planes<<<EXH_NUM_SMS * 16, 256, 0, st>>>(in, ng, out);
  count_launch(1);
  return cudaGetLastError() == cudaSuccess ? EXH_OK : EXH_E_CUDA;
}

int particles(const BoxParams& b, const float* S, const float* V, const HaloOut& o, float* pos, float* vel,
              cudaStream_t st) {
  const size_t sm = sizeof(float) * ((size_t)b.nd[0] + b.nd[1] + b.nd[2]);
  EXH_CUDA_TRY(set_smem(k_particles, sm));
  k_particles<<<EXH_NUM_SMS * 16, 256, sm, st>>>(S, V, b.nd[0], b.nd[1], b.nd[2], o, pos, vel);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

}  // namespace exh
