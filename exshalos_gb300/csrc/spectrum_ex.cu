// General tracer grids and power spectra: the options of grid_compute and
// power_compute beyond one unit-mass tracer type with CIC.
//
// grid   <- Tracer_Grid (src/spectrum/gridmodule.c:146-376) with NGP, CIC,
//           Sphere and Exp assignment (gridmodule.c:7-140), masses, several
//           tracer types, interlacing, the redshift-space shift and folding
// power  <- Power_Spectrum (src/spectrum/powermodule.c:4-108) over every
//           auto and cross spectrum of the types, Compute_gridk
//           (src/spectrum/spectrum_h.c:83-167) with interlacing and the
//           window of spectrum_h.c:51-70, Legendre multipoles up to l_max
//
// Assignment accumulates weight * mass / (mean mass) in 64-bit fixed point
// (quanta of 2^-40), so the grids do not depend on the order in which
// threads land; each tracer's deposited total is summed in FP64 for the
// normalisation grid / (M / ng) - 1.
#include <cmath>
#include <vector>

#include "ctx.cuh"
#include "fft4.cuh"
#include "spectrum.cuh"

namespace exh {

namespace {

constexpr double EX_Q = 1099511627776.0;       // 2^40
constexpr double EX_INV_Q = 1.0 / 1099511627776.0;
constexpr int EX_T = 256;
constexpr int EX_MAX_TYPES = 16;

__device__ __forceinline__ void ex_add(unsigned long long* g, double w) {
  atomicAdd(g, (unsigned long long)__double2ll_rn(w * EX_Q));
}

// cysumf of spectrum_h.c:17-27 with a bound on the turns
__device__ __forceinline__ float ex_wrap(float x, float L) {
  for (int it = 0; it < 1024 && x >= L; it++) x = __fsub_rn(x, L);
  for (int it = 0; it < 1024 && x < 0.f; it++) x = __fadd_rn(x, L);
  return x;
}

struct ExGridArgs {
  const float* pos;
  const float* vel;      // only with dir >= 0
  const float* mass;     // or null: unit masses
  const int* type;       // or null: one type
  int64_t np;
  int ntype, nd, window, inter, dir;
  float L, Ld, R, Rt, vfac;
  double inv_mbar;       // 1 / mean mass (1 without masses)
};

// deposit one tracer at post into acc (one grid); returns the deposited weight
__device__ double ex_deposit(const ExGridArgs& a, const float* post, double m, unsigned long long* acc) {
  const int nd = a.nd;
  const float Ld = a.Ld;
  int xt[3];
#pragma unroll
  for (int q = 0; q < 3; q++) {           // ind(), spectrum_h.c:73-80
    xt[q] = (int)floorf(__fdiv_rn(post[q], Ld));
    if (xt[q] >= nd) xt[q] = nd - 1;
    if (xt[q] < 0) xt[q] = 0;
  }
  const size_t n2 = (size_t)nd * nd;
  if (a.window == 1) {                    // NGP, gridmodule.c:7-14
    ex_add(&acc[xt[0] * n2 + (size_t)xt[1] * nd + xt[2]], m);
    return m;
  }
  if (a.window == 2) {                    // CIC, gridmodule.c:17-44
    float dx[3], t[3];
    int sg[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      float d = __fsub_rn(__fdiv_rn(post[q], Ld), (float)xt[q] + 0.5f);
      sg[q] = d >= 0.f ? 1 : -1;
      d = fabsf(d);
      dx[q] = d;
      t[q] = 1.f - d;
    }
    const int x1 = exh_wrap(xt[0], sg[0], nd), y1 = exh_wrap(xt[1], sg[1], nd), z1 = exh_wrap(xt[2], sg[2], nd);
    ex_add(&acc[xt[0] * n2 + (size_t)xt[1] * nd + xt[2]], m * (t[0] * t[1] * t[2]));
    ex_add(&acc[x1 * n2 + (size_t)xt[1] * nd + xt[2]], m * (dx[0] * t[1] * t[2]));
    ex_add(&acc[xt[0] * n2 + (size_t)y1 * nd + xt[2]], m * (t[0] * dx[1] * t[2]));
    ex_add(&acc[xt[0] * n2 + (size_t)xt[1] * nd + z1], m * (t[0] * t[1] * dx[2]));
    ex_add(&acc[x1 * n2 + (size_t)y1 * nd + xt[2]], m * (dx[0] * dx[1] * t[2]));
    ex_add(&acc[x1 * n2 + (size_t)xt[1] * nd + z1], m * (dx[0] * t[1] * dx[2]));
    ex_add(&acc[xt[0] * n2 + (size_t)y1 * nd + z1], m * (t[0] * dx[1] * dx[2]));
    ex_add(&acc[x1 * n2 + (size_t)y1 * nd + z1], m * (dx[0] * dx[1] * dx[2]));
    return m;
  }
  // Sphere (gridmodule.c:47-77) and Exp (gridmodule.c:80-113)
  const float Rr = a.window == 3 ? a.R : a.R * a.Rt;
  const int times = (int)floorf(0.5f + Rr / Ld);
  const float r2max = a.window == 3 ? __fmul_rn(a.R, a.R) : __fmul_rn(__fmul_rn(__fmul_rn(a.R, a.R), a.Rt), a.Rt);
  double M = 0.0;
  for (int i = -times; i <= times; i++) {
    const int ci = exh_wrap(xt[0], i % nd, nd);
    for (int j = -times; j <= times; j++) {
      const int cj = exh_wrap(xt[1], j % nd, nd);
      for (int k = -times; k <= times; k++) {
        const int ck = exh_wrap(xt[2], k % nd, nd);
        // float arithmetic of the reference, each operation rounded on its own
        float d[3] = {__fsub_rn(post[0], __fmul_rn((float)ci + 0.5f, Ld)),
                      __fsub_rn(post[1], __fmul_rn((float)cj + 0.5f, Ld)),
                      __fsub_rn(post[2], __fmul_rn((float)ck + 0.5f, Ld))};
#pragma unroll
        for (int q = 0; q < 3; q++) {
          if (d[q] > a.L / 2.f) d[q] = __fsub_rn(a.L, d[q]);
          if (d[q] < -a.L / 2.f) d[q] = __fadd_rn(a.L, d[q]);
        }
        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
        if (r2 <= r2max) {
          const double w = a.window == 3 ? m : m * (double)expf(-0.5f * r2 / a.R / a.R);
          ex_add(&acc[(size_t)ci * n2 + (size_t)cj * nd + ck], w);
          M += w;
        }
      }
    }
  }
  return M;
}

// one thread per tracer; per-block FP64 totals per grid
__global__ void __launch_bounds__(EX_T)
k_ex_assign(ExGridArgs a, unsigned long long* __restrict__ acc, double* __restrict__ part) {
  __shared__ double tot[2 * EX_MAX_TYPES];
  const int ngrid = a.ntype * (a.inter + 1);
  for (int q = threadIdx.x; q < ngrid; q += blockDim.x) tot[q] = 0.0;
  __syncthreads();
  const size_t ng = (size_t)a.nd * a.nd * a.nd;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.np; p += (int64_t)gridDim.x * blockDim.x) {
    const int ty = a.type ? a.type[p] : 0;
    if (ty < 0 || ty >= a.ntype) continue;
    const double m = a.mass ? (double)a.mass[p] * a.inv_mbar : 1.0;
    float post[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      float x = a.pos[3 * p + q];
      if (q == a.dir) x = __fadd_rn(x, __fmul_rn(a.vel[3 * p + q], a.vfac));    // gridmodule.c:167-170
      post[q] = ex_wrap(x, a.L);
    }
    const int g0 = ty * (a.inter + 1);
    const double m1 = ex_deposit(a, post, m, acc + (size_t)g0 * ng);
    atomicAdd(&tot[g0], m1);
    if (a.inter) {                        // the half-cell shifted grid, gridmodule.c:226-232
      float ps[3];
#pragma unroll
      for (int q = 0; q < 3; q++) ps[q] = ex_wrap(__fadd_rn(post[q], -a.Ld / 2.f), a.L);
      const double m2 = ex_deposit(a, ps, m, acc + (size_t)(g0 + 1) * ng);
      atomicAdd(&tot[g0 + 1], m2);
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < ngrid; q += blockDim.x) part[(size_t)blockIdx.x * ngrid + q] = tot[q];
}

// grid = (fixed-point sum) / (M / ng) - 1 for every grid
__global__ void k_ex_normalise(const unsigned long long* __restrict__ acc, size_t ng, int ngrid,
                               const double* __restrict__ Mtot, float* __restrict__ grid) {
  const size_t n = ng * (size_t)ngrid;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int gi = (int)(i / ng);
    const double rho = (double)(long long)acc[i] * EX_INV_Q;
    grid[i] = (float)(rho / (Mtot[gi] / (double)ng) - 1.0);
  }
}

// ------------------------------------------------------------------ power
struct ExPkArgs {
  int nd, nc, ntype, window, inter, Nk, ls, dir, nps;
  float kn, kmin, dk, Lb, R, Normk;
};

// window of spectrum_h.c:51-70
__device__ __forceinline__ float ex_window(const ExPkArgs& a, float kx, float ky, float kz) {
  auto sinc = [](float x) { return x != 0.f ? sinf(x) / x : 1.f; };
  switch (a.window) {
    case 1: return sinc(kx * a.Lb / 2.f) * sinc(ky * a.Lb / 2.f) * sinc(kz * a.Lb / 2.f);
    case 2: { const float w = sinc(kx * a.Lb / 2.f) * sinc(ky * a.Lb / 2.f) * sinc(kz * a.Lb / 2.f); return w * w; }
    case 3: {
      const float km = sqrtf(kx * kx + ky * ky + kz * kz);
      return 3.f / km / km / a.R / a.R * (sinc(km * a.R) - cosf(km * a.R));
    }
    case 4: return expf(-(kx * kx + ky * ky + kz * kz) * a.R * a.R / 2.f);
    default: return 1.f;
  }
}

// Compute_gridk: (X1 + X2 e^{-i (kx+ky+kz) Lb/2}) / 2 * Normk / W, or X1 Normk / W
__global__ void k_ex_gridk(const float2* __restrict__ X1, const float2* __restrict__ X2, ExPkArgs a,
                           float2* __restrict__ gk) {
  const size_t nk = (size_t)a.nd * a.nd * a.nc;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nk; t += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(t % a.nc);
    const size_t r = t / a.nc;
    const int j = (int)(r % a.nd), i = (int)(r / a.nd);
    const float kx = (float)((2 * i < a.nd) ? i : i - a.nd) * a.kn;
    const float ky = (float)((2 * j < a.nd) ? j : j - a.nd) * a.kn;
    const float kz = (float)((2 * k < a.nd) ? k : k - a.nd) * a.kn;
    const float s = a.Normk / ex_window(a, kx, ky, kz);
    const float2 o1 = X1[t];
    float2 v;
    if (X2) {
      const float2 o2 = X2[t];
      float sn, cs;
      sincosf((kx + ky + kz) * a.Lb / 2.f, &sn, &cs);
      v = make_float2((o1.x + o2.x * cs + o2.y * sn) / 2.f * s, (o1.y + o2.y * cs - o2.x * sn) / 2.f * s);
    } else {
      v = make_float2(o1.x * s, o1.y * s);
    }
    gk[t] = v;
  }
}

// every auto and cross spectrum and multipole: per-block FP64 histograms of
// [pair][multipole][bin], then k and counts
__global__ void __launch_bounds__(EX_T)
k_ex_bin(const float2* __restrict__ gk, ExPkArgs a, double* __restrict__ part) {
  extern __shared__ double hs[];
  const int nP = a.nps * a.ls * a.Nk;
  const int nh = nP + 2 * a.Nk;
  for (int b = threadIdx.x; b < nh; b += blockDim.x) hs[b] = 0.0;
  __syncthreads();
  const size_t nk = (size_t)a.nd * a.nd * a.nc;
  const int nd = a.nd;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nk; t += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(t % a.nc);
    const size_t r = t / a.nc;
    const int j = (int)(r % nd), i = (int)(r / nd);
    if ((k == 0 || k == nd / 2) &&
        ((i > nd / 2 && j > nd / 2) || i == 0 || i == nd / 2 || j == 0 || j == nd / 2 || (i > nd / 2 && j < nd / 2)))
      continue;                           // powermodule.c:50-51
    const float kx = (float)((2 * i < nd) ? i : i - nd) * a.kn;
    const float ky = (float)((2 * j < nd) ? j : j - nd) * a.kn;
    const float kz = (float)((2 * k < nd) ? k : k - nd) * a.kn;
    const float k2 = __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
    const float kmod = __fsqrt_rn(k2);
    const int bin = (int)floorf(__fdiv_rn(__fsub_rn(kmod, a.kmin), a.dk));
    if (bin < 0 || bin >= a.Nk) continue;
    float mu = 0.f;
    if (a.dir == 0) mu = kx / kmod;
    else if (a.dir == 1) mu = ky / kmod;
    else if (a.dir == 2) mu = kz / kmod;
    // Legendre P_0, P_2, P_4 ... by the three-term recurrence in FP64
    double leg[16];
    {
      const double x = (double)mu;
      double p0 = 1.0, p1 = x;
      leg[0] = 1.0;
      for (int l = 2; l <= 2 * (a.ls - 1); l++) {
        const double p2 = ((2.0 * l - 1.0) * x * p1 - (l - 1.0) * p0) / l;
        p0 = p1;
        p1 = p2;
        if ((l & 1) == 0) leg[l / 2] = p2;
      }
    }
    int pr = 0;
    for (int l = 0; l < a.ntype; l++) {
      const float2 gl = gk[(size_t)l * nk + t];
      for (int m = 0; m <= l; m++, pr++) {
        const float2 gm = gk[(size_t)m * nk + t];
        const double c = (double)(gl.x * gm.x + gl.y * gm.y);
        for (int n = 0; n < a.ls; n++) atomicAdd(&hs[(pr * a.ls + n) * a.Nk + bin], c * leg[n]);
      }
    }
    atomicAdd(&hs[nP + bin], (double)kmod);
    atomicAdd(&hs[nP + a.Nk + bin], 1.0);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nh; b += blockDim.x) part[(size_t)blockIdx.x * nh + b] = hs[b];
}

// fixed-order sum of the per-block histograms
__global__ void k_ex_reduce(const double* __restrict__ part, int nblk, int nh, double* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nh) return;
  double s = 0.0;
  for (int q = 0; q < nblk; q++) s += part[(size_t)q * nh + b];
  out[b] = s;
}

inline unsigned ex_blocks(size_t n) { return (unsigned)std::min<size_t>(exh_div_up(n, EX_T), (size_t)EXH_NUM_SMS * 8); }

}  // namespace

}  // namespace exh

using namespace exh;

#define EX_REQUIRE(cond, code, msg)                   \
  do {                                                \
    if (!(cond)) {                                    \
      exh_set_error_msg(msg, __FILE__, __LINE__);     \
      return code;                                    \
    }                                                 \
  } while (0)

extern "C" int exh_grid_compute_ex(exh_ctx* ctx, const float* pos, const float* vel, const float* mass,
                                   const int32_t* type, int64_t np, int ntype, int nd, float L, float Om0, float z,
                                   int direction, int window, float R, float R_times, int interlacing, int folds,
                                   float* grid, int mem, void* stream) {
  EX_REQUIRE(ctx && grid && (np == 0 || pos), EXH_E_INVALID, "null argument");
  EX_REQUIRE(np >= 0 && nd >= 2 && nd <= 1024 && L > 0.f && folds >= 1, EXH_E_INVALID,
             "need np >= 0, nd in [2, 1024], L > 0, folds >= 1");
  EX_REQUIRE(ntype >= 1 && ntype <= EX_MAX_TYPES, EXH_E_INVALID, "ntype must be in [1, 16]");
  EX_REQUIRE(window >= 1 && window <= 4, EXH_E_INVALID, "window must be 1 (NGP), 2 (CIC), 3 (Sphere) or 4 (Exp)");
  EX_REQUIRE(window < 3 || (R > 0.f && (window == 3 || R_times > 0.f)), EXH_E_INVALID, "Sphere/Exp need R > 0");
  EX_REQUIRE(direction >= -1 && direction <= 2 && (direction < 0 || vel), EXH_E_INVALID,
             "direction must be -1, 0, 1 or 2, with velocities for 0..2");
  EX_REQUIRE(ntype == 1 || type, EXH_E_INVALID, "several types need the type array");
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  const float Lf = L / (float)folds;                   // gridmodule.c:152-153
  const size_t ng = (size_t)nd * nd * nd;
  const int ngrid = ntype * (interlacing ? 2 : 1);
  // inputs on the device (staged in the context for host memory)
  const float *dpos = pos, *dvel = vel, *dmass = mass;
  const int* dtype = type;
  if (mem == EXH_MEM_HOST && np > 0) {
    size_t bytes = 12 * (size_t)np + 256;
    if (direction >= 0) bytes += 12 * (size_t)np + 256;
    if (mass) bytes += 4 * (size_t)np + 256;
    if (type) bytes += 4 * (size_t)np + 256;
    EXH_TRY(c.buf[B_HOSTIO].ensure(bytes));
    char* q = c.buf[B_HOSTIO].as<char>();
    auto stage = [&](const void* h, size_t n) -> char* {
      char* d = q;
      q += (n + 255) & ~size_t(255);
      return cudaMemcpyAsync(d, h, n, cudaMemcpyHostToDevice, st) == cudaSuccess ? d : nullptr;
    };
    dpos = reinterpret_cast<const float*>(stage(pos, 12 * (size_t)np));
    if (direction >= 0) dvel = reinterpret_cast<const float*>(stage(vel, 12 * (size_t)np));
    if (mass) dmass = reinterpret_cast<const float*>(stage(mass, 4 * (size_t)np));
    if (type) dtype = reinterpret_cast<const int*>(stage(type, 4 * (size_t)np));
    EX_REQUIRE(dpos && (direction < 0 || dvel) && (!mass || dmass) && (!type || dtype), EXH_E_CUDA,
               "staging the tracers failed");
  }
  ExGridArgs a{};
  a.pos = dpos; a.vel = dvel; a.mass = dmass; a.type = ntype > 1 ? dtype : nullptr; a.np = np;
  a.ntype = ntype; a.nd = nd; a.window = window; a.inter = interlacing ? 1 : 0; a.dir = direction;
  a.L = Lf; a.Ld = Lf / (float)nd; a.R = R; a.Rt = R_times;
  // pow(1+z, 3) / H(Om0, z), gridmodule.c:3-5,167-170
  a.vfac = (float)(std::pow(1.0 + (double)z, 3.0) / (100.0 * std::sqrt((double)Om0 * std::pow(1.0 + (double)z, 3.0) +
                                                                        (1.0 - (double)Om0))));
  a.inv_mbar = 1.0;
  const unsigned nb = ex_blocks((size_t)std::max<int64_t>(np, 1));
  EXH_TRY(c.buf[B_CICACC].ensure(sizeof(unsigned long long) * ng * ngrid));
  EXH_TRY(c.buf[B_SCRATCH].ensure(sizeof(double) * ((size_t)nb * ngrid + ngrid + 8)));
  unsigned long long* acc = c.buf[B_CICACC].as<unsigned long long>();
  double* part = c.buf[B_SCRATCH].as<double>();
  if (dmass && np > 0) {
    // mean mass in FP64 (the weights are accumulated relative to it)
    std::vector<float> hm;
    const float* msrc = mass;
    if (mem != EXH_MEM_HOST) {
      hm.resize(np);
      EXH_CUDA_TRY(cudaMemcpyAsync(hm.data(), mass, 4 * (size_t)np, cudaMemcpyDeviceToHost, st));
      EXH_CUDA_TRY(cudaStreamSynchronize(st));
      msrc = hm.data();
    }
    long double s = 0.0L;
    for (int64_t i = 0; i < np; i++) s += (long double)msrc[i];
    EX_REQUIRE(s > 0.0L, EXH_E_INVALID, "the total tracer mass must be positive");
    a.inv_mbar = (double)((long double)np / s);
  }
  EXH_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * ng * ngrid, st));
  if (np > 0) {
    KTimer kt(KC_CIC, st, 12.0 * np);
    k_ex_assign<<<nb, EX_T, 0, st>>>(a, acc, part);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  std::vector<double> hp((size_t)nb * ngrid, 0.0), Mt(ngrid, 0.0);
  if (np > 0) {
    EXH_CUDA_TRY(cudaMemcpyAsync(hp.data(), part, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
  }
  for (unsigned b = 0; b < nb; b++)
    for (int q = 0; q < ngrid; q++) Mt[q] += hp[(size_t)b * ngrid + q];
  double* dM = part + (size_t)nb * ngrid;
  if (sizeof(double) * ngrid <= UPLOAD_SMALL_MAX) {
    EXH_TRY(upload_small(dM, Mt.data(), sizeof(double) * ngrid, st));
  } else {
    EXH_CUDA_TRY(cudaMemcpyAsync(dM, Mt.data(), sizeof(double) * ngrid, cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));     // Mt dies at return
  }
  float* g = grid;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_GRID].ensure(sizeof(float) * ng * ngrid));
    g = c.buf[B_GRID].as<float>();
  }
  {
    KTimer kt(KC_CIC, st, 12.0 * ng * ngrid);
    k_ex_normalise<<<ex_blocks(ng * ngrid), EX_T, 0, st>>>(acc, ng, ngrid, dM, g);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  if (mem == EXH_MEM_HOST)
    EXH_CUDA_TRY(cudaMemcpyAsync(grid, g, sizeof(float) * ng * ngrid, cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  return EXH_OK;
}

extern "C" int exh_power_compute_ex(exh_ctx* ctx, const float* grid, int ntype, int nd, float L, int window,
                                    float R, int interlacing, int Nk, float k_min, float k_max, int l_max,
                                    int direction, float* k_out, float* P_out, int64_t* count_out, int mem,
                                    void* stream) {
  EX_REQUIRE(ctx && grid && k_out && P_out && count_out, EXH_E_INVALID, "null argument");
  EX_REQUIRE(nd >= 4 && nd <= 1024 && (nd % 2) == 0 && L > 0.f, EXH_E_INVALID, "nd must be even in [4, 1024], L > 0");
  EX_REQUIRE(ntype >= 1 && ntype <= EX_MAX_TYPES, EXH_E_INVALID, "ntype must be in [1, 16]");
  EX_REQUIRE(Nk >= 1 && Nk <= 4096 && k_max > k_min, EXH_E_INVALID, "need 1 <= Nk <= 4096 and k_max > k_min");
  EX_REQUIRE(window >= 0 && window <= 4 && (window < 3 || R > 0.f), EXH_E_INVALID,
             "window must be in 0..4 (3 and 4 need R > 0)");
  EX_REQUIRE(l_max >= 0 && l_max <= 30 && direction >= -1 && direction <= 2, EXH_E_INVALID,
             "need 0 <= l_max <= 30 and direction in -1..2");
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(nd, nd, nd, &p));
  const size_t ng = (size_t)nd * nd * nd, nk = (size_t)nd * nd * p->nc;
  const int ngrid = ntype * (interlacing ? 2 : 1);
  const float* g = grid;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_GRID].ensure(sizeof(float) * ng * ngrid));
    EXH_CUDA_TRY(cudaMemcpyAsync(c.buf[B_GRID].p, grid, sizeof(float) * ng * ngrid, cudaMemcpyHostToDevice, st));
    g = c.buf[B_GRID].as<float>();
  }
  ExPkArgs a{};
  a.nd = nd; a.nc = p->nc; a.ntype = ntype; a.window = window; a.inter = interlacing ? 1 : 0;
  a.Nk = Nk; a.ls = l_max / 2 + 1; a.dir = direction; a.nps = ntype * (ntype + 1) / 2;
  a.kn = (float)(2 * M_PI / L); a.kmin = k_min; a.dk = (k_max - k_min) / (float)Nk; a.Lb = L / (float)nd; a.R = R;
  a.Normk = (float)std::pow((double)(L / (float)(nd * nd)), 1.5);
  EX_REQUIRE(a.ls <= 16, EXH_E_INVALID, "l_max too large");
  // transformed grids: gk[ntype][nk], plus two work arrays
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  EXH_TRY(c.buf[B_WORK2].ensure(sizeof(float2) * nk * (ntype + 1)));
  c.mass_key.clear();                   // the mass tables of the halo finder share B_WORK2
  float2* w1 = c.buf[B_WORK].as<float2>();
  float2* w2 = c.buf[B_WORK2].as<float2>();
  float2* gk = w2 + nk;
  for (int l = 0; l < ntype; l++) {
    const float* g1 = g + (size_t)(l * (a.inter + 1)) * ng;
    EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{g1, nd}, w1, CplxStore{w1, nd, nd * p->nc}, st));
    const float2* x2 = nullptr;
    if (a.inter) {
      EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{g1 + ng, nd}, w2, CplxStore{w2, nd, nd * p->nc}, st));
      x2 = w2;
    }
    k_ex_gridk<<<ex_blocks(nk), EX_T, 0, st>>>(w1, x2, a, gk + (size_t)l * nk);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  const int nh = a.nps * a.ls * Nk + 2 * Nk;
  const size_t sm = sizeof(double) * nh;
  EX_REQUIRE(sm <= 200 * 1024, EXH_E_INVALID, "too many spectra x multipoles x bins for one block's histograms");
  const unsigned nb = EXH_NUM_SMS * 2;
  EXH_TRY(c.buf[B_SCRATCH].ensure(sizeof(double) * ((size_t)nb * nh + nh)));
  double* part = c.buf[B_SCRATCH].as<double>();
  double* tot = part + (size_t)nb * nh;
  EXH_CUDA_TRY(set_smem(k_ex_bin, sm));
  {
    KTimer kt(KC_BIN, st, 8.0 * nk * ntype);
    k_ex_bin<<<nb, EX_T, sm, st>>>(gk, a, part);
    k_ex_reduce<<<exh_div_up(nh, 256), 256, 0, st>>>(part, nb, nh, tot);
    count_launch(2);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  std::vector<double> h(nh);
  EXH_CUDA_TRY(cudaMemcpyAsync(h.data(), tot, sizeof(double) * nh, cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  const int nP = a.nps * a.ls * Nk;
  for (int i = 0; i < Nk; i++) {
    const double n = h[nP + Nk + i];
    count_out[i] = (int64_t)n;
    k_out[i] = n > 0 ? (float)(h[nP + i] / n) : 0.f;
    for (int q = 0; q < a.nps; q++)
      for (int m = 0; m < a.ls; m++) {
        const size_t o = ((size_t)q * a.ls + m) * Nk + i;
        P_out[o] = n > 0 ? (float)((4.0 * m + 1.0) * h[o] / n) : 0.f;      // powermodule.c:96-101
      }
  }
  return EXH_OK;
}
