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
#include "fft.cuh"
#include "field.cuh"
#include "halos.cuh"
#include "lpt.cuh"

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
__device__ __forceinline__ double d6(const float* __restrict__ f, size_t c, size_t sp1, size_t sp2, size_t sp3,
                                     size_t sm1, size_t sm2, size_t sm3) {
  return 1.0 * f[sp3] - 9.0 * f[sp2] + 45.0 * f[sp1] - 45.0 * f[sm1] + 9.0 * f[sm2] - 1.0 * f[sm3];
}

struct Nb {
  size_t p1, p2, p3, m1, m2, m3;
};
__device__ __forceinline__ Nb nb_axis(int i, int j, int k, int axis, int n0, int n1, int n2) {
  int c[3] = {i, j, k};
  const int n[3] = {n0, n1, n2};
  Nb r;
  size_t* out[6] = {&r.p1, &r.p2, &r.p3, &r.m1, &r.m2, &r.m3};
  const int off[6] = {1, 2, 3, -1, -2, -3};
#pragma unroll
  for (int t = 0; t < 6; t++) {
    int cc[3] = {c[0], c[1], c[2]};
    cc[axis] = exh_wrap(c[axis], off[t], n[axis]);
    *out[t] = ((size_t)cc[0] * n1 + cc[1]) * n2 + cc[2];
  }
  return r;
}

__device__ __forceinline__ double grad6(const float* __restrict__ f, int i, int j, int k, int axis, int n0, int n1,
                                        int n2) {
  const Nb b = nb_axis(i, j, k, axis, n0, n1, n2);
  return d6(f, 0, b.p1, b.p2, b.p3, b.m1, b.m2, b.m3);
}

// S1 for every cell, planes S[a * ng + cell]
__global__ void k_lpt1_disp(const float* __restrict__ phi, int n0, int n1, int n2, float fac, float* __restrict__ S) {
  const size_t ng = (size_t)n0 * n1 * n2;
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; c < ng; c += stride) {
    const int k = (int)(c % n2);
    const size_t r = c / n2;
    const int j = (int)(r % n1), i = (int)(r / n1);
#pragma unroll
    for (int a = 0; a < 3; a++) S[a * ng + c] = (float)(-grad6(phi, i, j, k, a, n0, n1, n2) * (double)fac);
  }
}

// second-order source (lpt.c:116-134)
__global__ void k_lpt2_source(const float* __restrict__ S, int n0, int n1, int n2, float inv60lc,
                              float* __restrict__ src) {
  const size_t ng = (size_t)n0 * n1 * n2;
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const float* Sx = S;
  const float* Sy = S + ng;
  const float* Sz = S + 2 * ng;
  for (; c < ng; c += stride) {
    const int k = (int)(c % n2);
    const size_t r = c / n2;
    const int j = (int)(r % n1), i = (int)(r / n1);
    const double l = (double)inv60lc;
    const float pxx = (float)(grad6(Sx, i, j, k, 0, n0, n1, n2) * l);
    const float pxy = (float)(grad6(Sx, i, j, k, 1, n0, n1, n2) * l);
    const float pxz = (float)(grad6(Sx, i, j, k, 2, n0, n1, n2) * l);
    const float pyy = (float)(grad6(Sy, i, j, k, 1, n0, n1, n2) * l);
    const float pyz = (float)(grad6(Sy, i, j, k, 2, n0, n1, n2) * l);
    const float pzz = (float)(grad6(Sz, i, j, k, 2, n0, n1, n2) * l);
    src[c] = (float)((double)(pxx * pyy + pxx * pzz + pyy * pzz) - (double)pxy * pxy - (double)pxz * pxz -
                     (double)pyz * pyz);
  }
}

// x pass of the 2LPT Poisson solve: forward, x Normk/(-k^2), inverse
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
    if (b < nb) {
      float kmod;
      const float s = g.k2(e, col / nc, col % nc, kmod);
      if (s == 0.f || kmod > g.k_smooth) v = make_float2(0.f, 0.f);
      else {
        const float f = -(kmod * kmod);
        v = make_float2(v.x / f * normk, v.y / f * normk);
      }
    }
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
// one warp per halo: sum of S1 (+ S2 from D6(phi2)) over member cells
__global__ void k_halo_disp(const int* __restrict__ hpeak, const int* __restrict__ gfin, const unsigned* __restrict__ pid,
                            int64_t np, int64_t nh, const int* __restrict__ off_all, const int* __restrict__ start_all,
                            const float* __restrict__ S, const float* __restrict__ phi2, int n0, int n1, int n2,
                            float s2fac, HaloOut o) {
  const int64_t h = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (h >= nh) return;
  const size_t ng = (size_t)n0 * n1 * n2;
  const int r = hpeak[h];
  const unsigned cell0 = pid[np - 1 - r];
  const int z0 = (int)(cell0 % n2);
  const unsigned rr = cell0 / n2;
  const int y0 = (int)(rr % n1), x0 = (int)(rr / n1);
  const int e = start_all[gfin[r]];
  double s1[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
  for (int q = lane; q < e; q += 32) {
    const int pk = off_all[q];
    const int i = exh_wrap(x0, (pk & 0xff) - 128, n0), j = exh_wrap(y0, ((pk >> 8) & 0xff) - 128, n1),
              k = exh_wrap(z0, ((pk >> 16) & 0xff) - 128, n2);
    const size_t c = ((size_t)i * n1 + j) * n2 + k;
#pragma unroll
    for (int a = 0; a < 3; a++) s1[a] += (double)S[a * ng + c];
    if (phi2) {
#pragma unroll
      for (int a = 0; a < 3; a++) s2[a] += (double)(float)(grad6(phi2, i, j, k, a, n0, n1, n2) * (double)s2fac);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) {
      s1[a] += __shfl_xor_sync(0xffffffffu, s1[a], w);
      s2[a] += __shfl_xor_sync(0xffffffffu, s2[a], w);
    }
  if (lane == 0) {
    const int cnt = e;
    const int xc[3] = {x0, y0, z0};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float disp = (float)(s1[a] + s2[a]);
      // cysumf(x Lc + Lc/2, disp/count, L) of lpt.c:245-255
      const float xq = (float)((double)((float)xc[a] * o.Lc) + (double)o.Lc / 2.0);
      float p = xq + disp / (float)cnt;
      if (p >= o.L[a]) p -= o.L[a];
      if (p < 0.f) p += o.L[a];
      o.posh[3 * h + a] = p;
      if (o.velh) o.velh[3 * h + a] = (float)((o.f1 * s1[a] + o.f2 * s2[a]) / (double)cnt);
    }
  }
}

// particle positions q + S1 + S2 and velocities for every cell (lpt.c:82-92,
// 212-222, 229-242); outputs interleaved [ng][3]
__global__ void k_particles(const float* __restrict__ S, const float* __restrict__ phi2, int n0, int n1, int n2,
                            float s2fac, HaloOut o, float* __restrict__ pos, float* __restrict__ vel) {
  const size_t ng = (size_t)n0 * n1 * n2;
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; c < ng; c += stride) {
    const int k = (int)(c % n2);
    const size_t r = c / n2;
    const int j = (int)(r % n1), i = (int)(r / n1);
    const int xc[3] = {i, j, k};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float s1 = S[a * ng + c];
      const float s2 = phi2 ? (float)(grad6(phi2, i, j, k, a, n0, n1, n2) * (double)s2fac) : 0.f;
      const float s = s1 + s2;
      const float xq = (float)((double)((float)xc[a] * o.Lc) + (double)o.Lc / 2.0);
      float p = xq + s;
      if (p >= o.L[a]) p -= o.L[a];
      if (p < 0.f) p += o.L[a];
      pos[3 * c + a] = p;
      if (vel) vel[3 * c + a] = (float)(o.f1 * s1 + o.f2 * s2);
    }
  }
}

int lpt_run(Ctx& c, const BoxParams& b, const FieldModes& modes, float k_smooth, bool do2, float* S, float* phi1,
            float* phi2, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
  const size_t nk = (size_t)b.nd[0] * b.nd[1] * p->nc;
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  float2* work = c.buf[B_WORK].as<float2>();
  KGrid g{b.nd[0], b.nd[1], b.nd[2], b.kl[0], b.kl[1], b.kl[2], k_smooth};
  EXH_CUDA_TRY(fft_c2r_3d(*p, Lpt1Gen{modes, g}, work, RealPairStore{phi1, b.nd[2], 1.f}, st));
  const unsigned grid = EXH_NUM_SMS * 16;
  { KTimer kt(KC_LPT_STENCIL, st, 16.0 * b.ng);
  k_lpt1_disp<<<grid, 256, 0, st>>>(phi1, b.nd[0], b.nd[1], b.nd[2], (float)(b.Normx / (60.0 * b.Lc)), S); }
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  if (!do2) return EXH_OK;
  float* src = phi2;   // the source is transformed, then phi2 overwrites it
  { KTimer kt(KC_LPT_STENCIL, st, 16.0 * b.ng);
  k_lpt2_source<<<grid, 256, 0, st>>>(S, b.nd[0], b.nd[1], b.nd[2], (float)(1.0 / (60.0 * b.Lc)), src); }
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  const size_t rows = (size_t)b.nd[0] * b.nd[1];
  EXH_CUDA_TRY(launch_r2c_rows(RealPairLoad{src, b.nd[2]}, HalfStore{work, p->nc}, *p, rows, st));
  EXH_CUDA_TRY(launch_strided(CplxLoad{work, b.nd[1], p->nc}, CplxStore{work, b.nd[1], p->nc}, p->py, p->twy, -1.f,
                              b.nd[0], p->nc, st));
  const int inner = b.nd[1] * p->nc;
  const size_t sm = smem_strided(b.nd[0]);
  EXH_CUDA_TRY(set_smem(k_fft_x_poisson, sm));
  { KTimer kt(KC_FFT_STRIDED, st, 16.0 * b.nd[0] * inner);
  k_fft_x_poisson<<<exh_div_up(inner, FFT_W), FFT_THREADS, sm, st>>>(work, p->px, p->twx, inner, g, b.Normk); }
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  EXH_CUDA_TRY(launch_strided(CplxLoad{work, b.nd[1], p->nc}, CplxStore{work, b.nd[1], p->nc}, p->py, p->twy, 1.f,
                              b.nd[0], p->nc, st));
  EXH_CUDA_TRY(launch_c2r_rows(HalfLoad{work, p->nc}, RealPairStore{phi2, b.nd[2], 1.f}, *p, rows, st));
  return EXH_OK;
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

int halo_displacements(Ctx& c, const BoxParams& b, const HaloDev& h, const ShellTable& t, const float* S,
                       const float* phi2, const HaloOut& o, cudaStream_t st) {
  (void)c;
  if (h.nh == 0) return EXH_OK;
  const int64_t threads = h.nh * 32;
  KTimer kt(KC_HALO_DISP, st, 0.0);
  k_halo_disp<<<exh_div_up(threads, 256), 256, 0, st>>>(h.hpeak, h.gfin, h.id, h.np, h.nh, t.off_all, t.start_all, S,
                                                        phi2, b.nd[0], b.nd[1], b.nd[2], lpt2_factor(b), o);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

int particles(const BoxParams& b, const float* S, const float* phi2, const HaloOut& o, float* pos, float* vel,
              cudaStream_t st) {
  k_particles<<<EXH_NUM_SMS * 16, 256, 0, st>>>(S, phi2, b.nd[0], b.nd[1], b.nd[2], lpt2_factor(b), o, pos, vel);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

}  // namespace exh
