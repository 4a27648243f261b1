// CIC density assignment and the shell-binned power spectrum.
//
// grid_compute   <- src/spectrum/spectrum.c:46-108, gridmodule.c:21-53,146-211
// power_compute  <- src/spectrum/spectrum.c:111-197, powermodule.c:4-108,
//                   spectrum_h.c:39-70,83-167
//
// The power spectrum never stores the transformed grid: the x pass of the
// real-to-complex FFT deconvolves the window and bins |delta_k|^2 straight
// from shared memory into per-block FP64 histograms.
#include <cmath>
#include <mutex>

#include "ctx.cuh"
#include "fft4.cuh"
#include "fixedpoint.cuh"
#include "fp32sum.cuh"
#include "spectrum.cuh"

namespace exh {

// ------------------------------------------------------------------ CIC
// One thread per tracer: the periodic wrap of spectrum_h.c:17-27, the cell
// index of spectrum_h.c:73-80 and the eight weights of gridmodule.c:29-50.
//
// The weights are accumulated in 64-bit fixed point (quanta of 2^-40, one
// rounding per weight) with integer atomics.  Integer addition is
// associative, so the grid does not depend on the order in which threads
// land: every run, every stream schedule and every batch gives the same
// bits.  Each cell is rounded to float once, from the exact fixed-point sum.
// Range: 2^23 tracers in one cell before the 64-bit sum overflows.  The
// conversions (round(w 2^40) in, (float)((double)sum 2^-40) out) run in
// integer arithmetic (fixedpoint.cuh), off the FP64 pipe.
__device__ __forceinline__ void cic_add(unsigned long long* g, float w) {
  atomicAdd(g, (unsigned long long)fp_quanta40(w));
}

__global__ void k_cic(const float* __restrict__ pos, int64_t np, int nd, float L, float Ld,
                      unsigned long long* __restrict__ acc) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  int xt[3], sg[3];
  float dx[3], t[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    float x = pos[3 * p + a];
    // at most a few turns for finite input; non-finite input is left alone
    for (int it = 0; it < 64 && x >= L; it++) x = __fsub_rn(x, L);
    for (int it = 0; it < 64 && x < 0.f; it++) x = __fadd_rn(x, L);
    if (!(x >= 0.f && x < L)) return;
    const float q = __fdiv_rn(x, Ld);
    int c = (int)floorf(q);
    if (c >= nd) c = nd - 1;
    xt[a] = c;
    float d = __fsub_rn(q, (float)c + 0.5f);
    if (d >= 0.f) { sg[a] = 1; }
    else { sg[a] = -1; d = -d; }
    dx[a] = d;
    t[a] = __fsub_rn(1.f, d);
  }
  const int x0 = xt[0], y0 = xt[1], z0 = xt[2];
  const int x1 = exh_wrap(x0, sg[0], nd), y1 = exh_wrap(y0, sg[1], nd), z1 = exh_wrap(z0, sg[2], nd);
  const size_t n2 = (size_t)nd * nd;
  cic_add(&acc[x0 * n2 + (size_t)y0 * nd + z0], t[0] * t[1] * t[2]);
  cic_add(&acc[x1 * n2 + (size_t)y0 * nd + z0], dx[0] * t[1] * t[2]);
  cic_add(&acc[x0 * n2 + (size_t)y1 * nd + z0], t[0] * dx[1] * t[2]);
  cic_add(&acc[x0 * n2 + (size_t)y0 * nd + z1], t[0] * t[1] * dx[2]);
  cic_add(&acc[x1 * n2 + (size_t)y1 * nd + z0], dx[0] * dx[1] * t[2]);
  cic_add(&acc[x1 * n2 + (size_t)y0 * nd + z1], dx[0] * t[1] * dx[2]);
  cic_add(&acc[x0 * n2 + (size_t)y1 * nd + z1], t[0] * dx[1] * dx[2]);
  cic_add(&acc[x1 * n2 + (size_t)y1 * nd + z1], dx[0] * dx[1] * dx[2]);
}

// rho = fixed-point sum rounded to float; delta = rho / (np / ng) - 1
// (gridmodule.c:206-211)
__global__ void k_cic_normalise(const unsigned long long* __restrict__ acc, float* __restrict__ grid, size_t ng,
                                float inv_mean) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < ng; i += stride) {
    const float rho = fp_value40(acc[i]);
    grid[i] = rho * inv_mean - 1.f;
  }
}

int cic_assign(Ctx& c, const float* pos_dev, int64_t np, int nd, float L, float* grid_dev, cudaStream_t st) {
  const size_t ng = (size_t)nd * nd * nd;
  EXH_TRY(c.buf[B_CICACC].ensure(sizeof(unsigned long long) * ng));
  unsigned long long* acc = c.buf[B_CICACC].as<unsigned long long>();
  EXH_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * ng, st));
  const float Ld = L / (float)nd;
  if (np > 0) {
    KTimer kt(KC_CIC, st, 12.0 * np + 64.0 * np);
    k_cic<<<exh_div_up(np, 256), 256, 0, st>>>(pos_dev, np, nd, L, Ld, acc);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  // np == 0 gives 0/0 in the reference; the grid is returned as -1 + nan there.
  const float inv_mean = np > 0 ? (float)((double)ng / (double)np) : NAN;
  { KTimer kt(KC_CIC, st, 12.0 * ng);
  k_cic_normalise<<<EXH_NUM_SMS * 8, 256, 0, st>>>(acc, grid_dev, ng, inv_mean); }
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

// ------------------------------------------------------------------ P(k)
__device__ __forceinline__ float sinc_f(float x) { return x != 0.f ? sinf(x) / x : 1.f; }

// A run of same-bin modes is summed in a compensated float sum (FSum) and
// goes to the double histogram as its exact hi + lo.
using RunSum = FSum;

// Binning of one transformed tile res[i * W + b] (x index i < n, column
// b < nb of the tile starting at inner index i0) into the block's shared
// histograms.
__device__ __forceinline__ void bin_tile(const float2* res, int W, int n, int nb, int i0, int nd, int nc,
                                         const BinParams& bp, double* hP, double* hK, unsigned* hN) {
  // one thread per x row of the tile walks its W adjacent (y, kz)
  // columns (cyclically, from a per-row start); neighbouring kz mostly share
  // a shell, so the thread adds a run of same-bin modes in registers and
  // touches the shared histogram once per run
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int cur = -1;
    RunSum aP, aK;
    unsigned aN = 0u;
    for (int bb = 0; bb < nb; bb++) {
      const int b = (bb + i) % nb;          // staggered start: rows of a warp hit different banks
      const int col = i0 + b, j = col / nc, k = col % nc;
      // mode-skip rule of powermodule.c:50-51 on the kz = 0 and kz = nd/2 planes
      if ((k == 0 || k == nd / 2) &&
          ((i > nd / 2 && j > nd / 2) || i == 0 || i == nd / 2 || j == 0 || j == nd / 2 || (i > nd / 2 && j < nd / 2)))
        continue;
      // wave numbers and bin index in the reference's float arithmetic
      const float kx = (float)((2 * i < nd) ? i : i - nd) * bp.kn;
      const float ky = (float)((2 * j < nd) ? j : j - nd) * bp.kn;
      const float kz = (float)((2 * k < nd) ? k : k - nd) * bp.kn;
      const float k2 = __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(ky, ky)), __fmul_rn(kz, kz));
      const float kmod = __fsqrt_rn(k2);
      const int bin = (int)floorf(__fdiv_rn(__fsub_rn(kmod, bp.kmin), bp.dk));
      if (bin < 0 || bin >= bp.Nk) continue;
      float w = 1.f;
      if (bp.window == 1 || bp.window == 2) {
        w = sinc_f(kx * bp.Lb * 0.5f) * sinc_f(ky * bp.Lb * 0.5f) * sinc_f(kz * bp.Lb * 0.5f);
        if (bp.window == 2) w = w * w;
      }
      // the deconvolved mode and its power in float, as the reference forms
      // them (gridk = out Normk / W, spectrum_h.c:161-162; re^2 + im^2,
      // powermodule.c:66); only the sums are wider
      const float2 v = res[i * W + b];
      const float re = __fdiv_rn(__fmul_rn(v.x, bp.Normk), w);
      const float im = __fdiv_rn(__fmul_rn(v.y, bp.Normk), w);
      const float pw = __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
      if (bin != cur) {
        if (cur >= 0) {
          atomicAdd(&hP[cur], aP.value());
          atomicAdd(&hK[cur], aK.value());
          atomicAdd(&hN[cur], aN);
        }
        cur = bin;
        aP = RunSum();
        aK = RunSum();
        aN = 0u;
      }
      aP.add(pw);
      aK.add(kmod);
      aN++;
    }
    if (cur >= 0) {
      atomicAdd(&hP[cur], aP.value());
      atomicAdd(&hK[cur], aK.value());
      atomicAdd(&hN[cur], aN);
    }
  }
}

// ---------------------------------------------------------------------------
// Binning epilogue of the four-step x passes (k_fft4_x_bin, k_fft8_x_bin512;
// Nk <= BINW_MAX_NK).  Same modes, wave numbers, |k| and bins as bin_tile,
// bit for bit, with only float work per mode:
// * rows i and nd - i have the same kx^2, hence the same |k|, bin and window
//   for every column: one lane takes the entry q = |kx| / kn, both its rows;
// * for a fixed column the bin is monotone in q (every step from q to the
//   bin is a monotone rounded operation), and the modes the reference skips
//   (powermodule.c:50-51) or that fall outside the bins sit at the ends of the
//   q order, so among 32 consecutive entries equal bins are contiguous: a warp
//   takes one column of 32 entries per step and sums each run of equal bins
//   with a segmented shuffle reduction; the run's first lane adds the sums to
//   the warp's histogram (float pairs (s, c) per bin, distinct bins within a
//   warp, no atomics) and the mode count to the block's (integer atomics);
// * the bin floor((|k| - kmin) / dk) is taken from (|k| - kmin) * (1/dk),
//   whose relative distance to the correctly rounded quotient is below 2^-22;
//   within BIN_EDGE of an integer the quotient is formed exactly (__fdiv_rn);
// * the window is separable: Normk / W = (Normk / wx) * (1 / (wy wz)), a
//   factor per entry and one per column, instead of two divisions per mode
//   (a few float ulps from the reference's gridk = out Normk / W);
// * the warps' histograms are combined per bin in float pairs (fixed order)
//   and turned into double once per bin and block.
// The tile is read as res[i * PW + b] with a padded row stride PW = W + 1, so
// the 32 entries of one column fall in distinct bank pairs.
constexpr int BINW_MAX_NK = 256;
constexpr float BIN_EDGE = 1.f / 2048.f;     // covers the 2^-22 relative gap for quotients below 2048

// (s, c) += hi + lo, s updated by an error-free TwoSum
__device__ __forceinline__ void pair_add(float& s, float& c, float hi, float lo) {
  const float t = __fadd_rn(s, hi);
  const float bb = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(hi, bb));
  s = t;
  c = __fadd_rn(c, __fadd_rn(e, lo));
}

// shared memory of the epilogue: a float4 per column (ky, kz, column factor,
// skip flags), 4 NW Nk floats (warp histograms), a float per entry (entry
// factor), 16 bytes of alignment slack
__host__ __device__ __forceinline__ size_t binw_smem(int NW, int Nk, int nd, int W) {
  return 16 + 16 * (size_t)W + sizeof(float) * (4 * (size_t)NW * Nk + (size_t)(nd / 2 + 2));
}

// The epilogue in three steps, for blocks that bin several tiles in turn:
// binw_begin once per block (warp histograms zeroed, the per-entry factors),
// binw_tile per tile (after a barrier: the tile in res; ends before the
// block's next barrier), binw_end once (after a barrier: the warp
// histograms combined into hP, hK).
struct BinwSmem {
  float4* colt;      // per column of the tile: ky, kz, column factor, skip flags
  float* ws;         // 4 NW Nk: the warps' (P sum, P carry, K sum, K carry)
  float* rowt;       // per entry q: Normk over the entry's window factor
  size_t stride;     // NW Nk
};

__device__ __forceinline__ BinwSmem binw_layout(void* scratch, int W, int Nk) {
  BinwSmem s;
  s.colt = reinterpret_cast<float4*>((reinterpret_cast<uintptr_t>(scratch) + 15) & ~(uintptr_t)15);
  s.ws = reinterpret_cast<float*>(s.colt + W);
  s.stride = (size_t)(blockDim.x >> 5) * Nk;
  s.rowt = s.ws + 4 * s.stride;
  return s;
}

__device__ void binw_begin(const BinwSmem& s, int nd, const BinParams& bp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Nk = bp.Nk, E = nd / 2 + 1;
  const int wq = bp.window == 2 ? 2 : (bp.window == 1 ? 1 : 0);     // W = (wx wy wz)^wq
  float* Ps = s.ws + (size_t)warp * Nk;
  for (int b = lane; b < Nk; b += 32) {
    Ps[b] = 0.f;
    Ps[s.stride + b] = 0.f;
    Ps[2 * s.stride + b] = 0.f;
    Ps[3 * s.stride + b] = 0.f;
  }
  for (int q = threadIdx.x; q < E; q += blockDim.x) {
    float rf = bp.Normk;
    if (wq) {
      float sn = sinc_f((float)q * bp.kn * bp.Lb * 0.5f);            // sinc is even: both rows of the entry
      if (wq == 2) sn = __fmul_rn(sn, sn);
      rf = __fdiv_rn(bp.Normk, sn);
    }
    s.rowt[q] = rf;
  }
}

__device__ void binw_tile(const BinwSmem& s, const float2* res, int PW, int nb, int i0, int nd, int nc,
                          const BinParams& bp, unsigned* hN) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, NW = blockDim.x >> 5;
  const int Nk = bp.Nk, h = nd / 2, E = h + 1, G = (E + 31) >> 5;
  const int wq = bp.window == 2 ? 2 : (bp.window == 1 ? 1 : 0);
  float* Ps = s.ws + (size_t)warp * Nk;
  float* Pc = Ps + s.stride;
  float* Ks = Pc + s.stride;
  float* Kc = Ks + s.stride;
  for (int t = threadIdx.x; t < nb; t += blockDim.x) {
    const int col = i0 + t, j = col / nc, k = col % nc;
    const float ky = (float)((2 * j < nd) ? j : j - nd) * bp.kn;
    const float kz = (float)((2 * k < nd) ? k : k - nd) * bp.kn;
    float cf = 1.f;
    if (wq) {
      float sn = __fmul_rn(sinc_f(ky * bp.Lb * 0.5f), sinc_f(kz * bp.Lb * 0.5f));
      if (wq == 2) sn = __fmul_rn(sn, sn);
      cf = __frcp_rn(sn);
    }
    const int flag = ((k == 0 || k == h) ? 1 : 0) | ((j == 0 || j == h) ? 2 : 0);
    s.colt[t] = make_float4(ky, kz, cf, __int_as_float(flag));
  }
  __syncthreads();
  const float inv_dk = __frcp_rn(bp.dk);
  const int units = G * nb;
  for (int u = warp; u < units; u += NW) {              // warp-uniform: (entry group, column)
    const int g = u / nb, b = u - g * nb;
    const int q = (g << 5) + lane;
    int key = -1, two = 0;
    float pw = 0.f, kk = 0.f;
    if (q < E) {
      const float4 cq = s.colt[b];
      const int fl = __float_as_int(cq.w);
      const bool fk = fl & 1, fj = fl & 2;
      const int r2 = nd - q;                            // the mirror row, when it is a row other than q
      const bool keep1 = !fk || (!fj && q > 0 && q < h);
      const bool keep2 = q > 0 && r2 > h && !fk;        // rows past nd/2 are skipped on the kz = 0, nd/2 planes
      if (keep1 || keep2) {
        const float kx = (float)q * bp.kn;              // (-q kn)^2 = (q kn)^2: the mirror row's kx^2
        const float k2 = __fadd_rn(__fadd_rn(__fmul_rn(kx, kx), __fmul_rn(cq.x, cq.x)), __fmul_rn(cq.y, cq.y));
        const float kmod = __fsqrt_rn(k2);
        const float d = __fsub_rn(kmod, bp.kmin);
        const float qf = __fmul_rn(d, inv_dk);
        float fb = floorf(qf);
        const float fr = __fsub_rn(qf, fb);
        if (fr <= BIN_EDGE || fr >= 1.f - BIN_EDGE) fb = floorf(__fdiv_rn(d, bp.dk));
        if (fb >= 0.f && fb < (float)Nk) {
          key = (int)fb;
          const float sc = __fmul_rn(s.rowt[q], cq.z);
          float p = 0.f;
          if (keep1) {
            const float2 v = res[q * PW + b];
            const float re = __fmul_rn(v.x, sc), im = __fmul_rn(v.y, sc);
            p = __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
          }
          if (keep2) {
            const float2 v = res[r2 * PW + b];
            const float re = __fmul_rn(v.x, sc), im = __fmul_rn(v.y, sc);
            p = __fadd_rn(p, __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im)));
          }
          pw = p;
          two = keep1 && keep2;
          kk = two ? __fadd_rn(kmod, kmod) : kmod;
        }
      }
    }
    const unsigned vmask = __ballot_sync(FULL, key >= 0);
    if (vmask == 0u) continue;
    const int kprev = __shfl_up_sync(FULL, key, 1);
    const bool start = key >= 0 && (lane == 0 || kprev != key);
    const unsigned bmask = __ballot_sync(FULL, start) | ~vmask;        // lanes where a run begins or breaks
    const unsigned above = bmask & (0xfffffffeu << lane);
    const int end = above ? __ffs(above) - 1 : 32;                    // one past this lane's run
    const unsigned tmask = __ballot_sync(FULL, two);
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {                             // suffix sums within the run
      const float tp = __shfl_down_sync(FULL, pw, dd), tk = __shfl_down_sync(FULL, kk, dd);
      if (lane + dd < end) {
        pw = __fadd_rn(pw, tp);
        kk = __fadd_rn(kk, tk);
      }
    }
    if (start) {
      const unsigned run = (end == 32 ? FULL : ((1u << end) - 1u)) & (FULL << lane);
      pair_add(Ps[key], Pc[key], pw, 0.f);
      pair_add(Ks[key], Kc[key], kk, 0.f);
      atomicAdd(&hN[key], (unsigned)(end - lane) + (unsigned)__popc(tmask & run));
    }
  }
}

__device__ void binw_end(const BinwSmem& s, int Nk, double* hP, double* hK) {
  const int NW = blockDim.x >> 5;
  for (int b = threadIdx.x; b < Nk; b += blockDim.x) {
    float ps = 0.f, pc = 0.f, ks = 0.f, kc = 0.f;
    for (int w = 0; w < NW; w++) {
      const size_t o = (size_t)w * Nk + b;
      pair_add(ps, pc, s.ws[o], s.ws[s.stride + o]);
      pair_add(ks, kc, s.ws[2 * s.stride + o], s.ws[3 * s.stride + o]);
    }
    hP[b] = (double)ps + (double)pc;
    hK[b] = (double)ks + (double)kc;
  }
}

// x pass of the forward transform with the binning epilogue.
// Tile: all nx modes of FFT_W adjacent (y, kz) columns.
__global__ void __launch_bounds__(FFT_THREADS)
k_fft_x_bin(const float2* __restrict__ work, RadixPlan pl, const float2* __restrict__ tw, int nd, int nc,
            BinParams bp, double* __restrict__ partP, double* __restrict__ partK,
            unsigned int* __restrict__ partN) {
  extern __shared__ float2 smem[];
  const int n = pl.n;
  float2* b0 = smem;
  float2* b1 = smem + n * FFT_W;
  double* hP = reinterpret_cast<double*>(smem + 2 * n * FFT_W);
  double* hK = hP + bp.Nk;
  unsigned int* hN = reinterpret_cast<unsigned int*>(hK + bp.Nk);
  const int inner = nd * nc;
  const int i0 = blockIdx.x * FFT_W;
  const int nb = min(FFT_W, inner - i0);
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) { hP[b] = 0.0; hK[b] = 0.0; hN[b] = 0u; }
  for (int t = threadIdx.x; t < n * FFT_W; t += blockDim.x) {
    const int e = t / FFT_W, b = t % FFT_W;
    b0[e * FFT_W + b] = (b < nb) ? work[(size_t)e * inner + i0 + b] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* res = stockham_run(b0, b1, pl, FFT_W, FFT_W, tw, -1.f);
  bin_tile(res, FFT_W, n, nb, i0, nd, nc, bp, hP, hK, hN);
  __syncthreads();
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) {
    partP[(size_t)blockIdx.x * bp.Nk + b] = hP[b];
    partK[(size_t)blockIdx.x * bp.Nk + b] = hK[b];
    partN[(size_t)blockIdx.x * bp.Nk + b] = hN[b];
  }
}

// The same x pass as a four-step register FFT (fft4.cuh) for the lengths it
// covers: step 1 and the transpose as k_fft4_strided, then the results go
// back to shared memory in natural order for the binning.  One tile per
// block: at these lengths the epilogue's set-up and combine are small beside
// the tile, and blocks that bin several tiles in turn (k_fft8_x_bin512) run
// slower here (fewer resident warps, no overlap of one block's loads with
// another's binning).
template <int N1, int N2>
__global__ void __launch_bounds__(FS_THREADS, 4)
k_fft4_x_bin(const float2* __restrict__ work, const float2* __restrict__ tw, int nd, int nc, BinParams bp,
             double* __restrict__ partP, double* __restrict__ partK, unsigned int* __restrict__ partN) {
  using S = FsShape<N1, N2>;
  constexpr int W = S::W, n = S::n;
  extern __shared__ float2 dsm[];
  float2* sm = dsm;
  double* hP = reinterpret_cast<double*>(sm + n * (W + 1));
  double* hK = hP + bp.Nk;
  unsigned int* hN = reinterpret_cast<unsigned int*>(hK + bp.Nk);
  const int inner = nd * nc;
  const int i0 = blockIdx.x * W;
  const int nb = min(W, inner - i0);
  const int c = threadIdx.x % W, jj = threadIdx.x / W;
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) { hP[b] = 0.0; hK[b] = 0.0; hN[b] = 0u; }
  if (jj < N2) {
    float2 v[N1];
#pragma unroll
    for (int j1 = 0; j1 < N1; j1++)
      v[j1] = (c < nb) ? work[(size_t)(jj + N2 * j1) * inner + i0 + c] : make_float2(0.f, 0.f);
    RDft<N1>::run(v, -1.f, [tw](int m) { return __ldg(&tw[m * N2]); });
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) {
      float2 x = v[k1];
      if (k1 != 0 && jj != 0) x = cmul(x, tw_get(tw, jj * k1, -1.f));
      sm[(k1 * N2 + jj) * W + c] = x;
    }
  }
  __syncthreads();
  float2 u[N2];
  if (jj < N1) {
#pragma unroll
    for (int j2 = 0; j2 < N2; j2++) u[j2] = sm[(jj * N2 + j2) * W + c];
    RDft<N2>::run(u, -1.f, [tw](int m) { return __ldg(&tw[m * N1]); });
  }
  __syncthreads();
  if (jj < N1) {
#pragma unroll
    for (int k2 = 0; k2 < N2; k2++) sm[(jj + N1 * k2) * (W + 1) + c] = u[k2];
  }
  if (bp.Nk <= BINW_MAX_NK) {
    const BinwSmem bs = binw_layout(hN + bp.Nk, W, bp.Nk);
    binw_begin(bs, nd, bp);
    __syncthreads();
    binw_tile(bs, sm, W + 1, nb, i0, nd, nc, bp, hN);
    __syncthreads();
    binw_end(bs, bp.Nk, hP, hK);
  } else {
    __syncthreads();
    bin_tile(sm, W + 1, n, nb, i0, nd, nc, bp, hP, hK, hN);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) {
    partP[(size_t)blockIdx.x * bp.Nk + b] = hP[b];
    partK[(size_t)blockIdx.x * bp.Nk + b] = hK[b];
    partN[(size_t)blockIdx.x * bp.Nk + b] = hN[b];
  }
}

// Length 512: the three radix-8 stages of k_fft8_strided512, the results
// back in shared memory in natural order for the binning.  Each block bins
// the tiles blockIdx.x * per .. + per - 1 in turn into one set of
// histograms: with 8-column tiles and up to 256 bins the per-tile histogram
// set-up, combine and partial sums cost as much as the tile itself (16448
// tiles wrote 73 MB of partials at 512^3), so they are paid once per block.
__global__ void __launch_bounds__(F512_T, 2)
k_fft8_x_bin512(const float2* __restrict__ work, const float2* __restrict__ tw, int nd, int nc, BinParams bp,
                int per, double* __restrict__ partP, double* __restrict__ partK, unsigned int* __restrict__ partN) {
  constexpr int W = F512_W, n = 512;
  extern __shared__ float2 dsm[];
  float2* sm = dsm;                                   // (n + 64) W float2
  double* hP = reinterpret_cast<double*>(sm + (n + 64) * W);
  double* hK = hP + bp.Nk;
  unsigned int* hN = reinterpret_cast<unsigned int*>(hK + bp.Nk);
  const int inner = nd * nc, ntile = (inner + W - 1) / W;
  const int c = threadIdx.x % W, q = threadIdx.x / W;
  const bool mirror = bp.Nk <= BINW_MAX_NK;
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) { hP[b] = 0.0; hK[b] = 0.0; hN[b] = 0u; }
  BinwSmem bs{};
  if (mirror) {
    bs = binw_layout(hN + bp.Nk, W, bp.Nk);
    binw_begin(bs, nd, bp);
  }
  const int t1 = min(ntile, (int)(blockIdx.x + 1) * per);
  for (int t = blockIdx.x * per; t < t1; t++) {
    const int i0 = t * W, nb = min(W, inner - i0);
    float2 v[8];
    f512_run([&](int j) { return (c < nb) ? work[(size_t)j * inner + i0 + c] : make_float2(0.f, 0.f); }, sm, tw,
             -1.f, c, q, v);
    __syncthreads();
    {
      const int k1 = q >> 3, k2a = q & 7;
#pragma unroll
      for (int k2b = 0; k2b < 8; k2b++) sm[(k1 + 8 * k2a + 64 * k2b) * (W + 1) + c] = v[k2b];
    }
    __syncthreads();
    if (mirror) binw_tile(bs, sm, W + 1, nb, i0, nd, nc, bp, hN);
    else bin_tile(sm, W + 1, n, nb, i0, nd, nc, bp, hP, hK, hN);
    __syncthreads();                                  // the tile and its columns are free again
  }
  if (mirror) binw_end(bs, bp.Nk, hP, hK);
  __syncthreads();
  for (int b = threadIdx.x; b < bp.Nk; b += blockDim.x) {
    partP[(size_t)blockIdx.x * bp.Nk + b] = hP[b];
    partK[(size_t)blockIdx.x * bp.Nk + b] = hK[b];
    partN[(size_t)blockIdx.x * bp.Nk + b] = hN[b];
  }
}

// Tiles per block for a binning x pass of ntile tiles: as many blocks as fit
// on the GPU at once (one wave), each with an equal share of the tiles.
template <class K>
static cudaError_t bin_blocks(K kernel, int threads, size_t smem, int ntile, int* per, int* grid) {
  int fit = 0;
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kernel, threads, smem);
  if (e != cudaSuccess) return e;
  const int resident = (fit > 0 ? fit : 1) * EXH_NUM_SMS;
  *per = (ntile + resident - 1) / resident;
  *grid = (ntile + *per - 1) / *per;
  return cudaSuccess;
}

// launches k_fft4_x_bin (k_fft8_x_bin512 for 512) for the lengths with a
// four-step split; returns the block count through nblk (0: not covered)
static cudaError_t launch_fs_x_bin(const float2* work, const float2* tw, int nd, int nc, const BinParams& bp,
                                   double* partP, double* partK, unsigned* partN, int nblk_cap, int* nblk,
                                   cudaStream_t st) {
  *nblk = 0;
  const int inner = nd * nc;
  if (nd == 512) {
    const int ntile = (int)exh_div_up(inner, F512_W);
    size_t sm = sizeof(float2) * (512 + 64) * F512_W + (size_t)bp.Nk * (2 * sizeof(double) + sizeof(unsigned)) + 16;
    if (bp.Nk <= BINW_MAX_NK) sm += binw_smem(F512_T / 32, bp.Nk, 512, F512_W);
    cudaError_t e = set_smem(k_fft8_x_bin512, sm);
    if (e != cudaSuccess) return e;
    int per = 0, nb = 0;
    e = bin_blocks(k_fft8_x_bin512, F512_T, sm, ntile, &per, &nb);
    if (e != cudaSuccess) return e;
    if (nb > nblk_cap) return cudaSuccess;
    k_fft8_x_bin512<<<nb, F512_T, sm, st>>>(work, tw, nd, nc, bp, per, partP, partK, partN);
    *nblk = nb;
    return cudaGetLastError();
  }
  switch (fs_split(nd)) {
#define X(A_, B_)                                                                                        \
  case A_ * 1000 + B_: {                                                                                 \
    using S = FsShape<A_, B_>;                                                                           \
    const int ntile = (int)exh_div_up(inner, S::W);                                                      \
    size_t sm = sizeof(float2) * S::n * (S::W + 1) + (size_t)bp.Nk * (2 * sizeof(double) + sizeof(unsigned)) + 16; \
    if (bp.Nk <= BINW_MAX_NK) sm += binw_smem(FS_THREADS / 32, bp.Nk, S::n, S::W);                      \
    cudaError_t e = set_smem(k_fft4_x_bin<A_, B_>, sm);                                                  \
    if (e != cudaSuccess) return e;                                                                      \
    if (ntile > nblk_cap) return cudaSuccess;                                                            \
    k_fft4_x_bin<A_, B_><<<ntile, FS_THREADS, sm, st>>>(work, tw, nd, nc, bp, partP, partK, partN);       \
    *nblk = ntile;                                                                                       \
    return cudaGetLastError();                                                                           \
  }
    EXH_FS_STRIDED_CASES(X)
#undef X
    default: return cudaSuccess;
  }
}

// per-bin sums over blocks, fixed order
__global__ void k_bin_reduce(const double* __restrict__ partP, const double* __restrict__ partK,
                             const unsigned int* __restrict__ partN, int nblk, int Nk, double* __restrict__ outP,
                             double* __restrict__ outK, long long* __restrict__ outN) {
  const int b = blockIdx.x;
  double sP = 0.0, sK = 0.0;
  unsigned long long sN = 0;
  for (int q = threadIdx.x; q < nblk; q += blockDim.x) {
    sP += partP[(size_t)q * Nk + b];
    sK += partK[(size_t)q * Nk + b];
    sN += partN[(size_t)q * Nk + b];
  }
  __shared__ double rP[256], rK[256];
  __shared__ unsigned long long rN[256];
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
    const unsigned long long n = rN[0];
    outN[b] = (long long)n;
    outP[b] = n ? rP[0] / (double)n : 0.0;     // (4l+1) = 1 for l = 0
    outK[b] = n ? rK[0] / (double)n : 0.0;
  }
}

int power_spectrum(Ctx& c, const float* grid_dev, int nd, float L, int window, int Nk, float kmin, float kmax,
                   double* outP_dev, double* outK_dev, long long* outN_dev, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(nd, nd, nd, &p));
  const size_t nk = (size_t)nd * nd * p->nc;
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  float2* work = c.buf[B_WORK].as<float2>();
  // z and y passes of the forward transform
  const size_t rows = (size_t)nd * nd;
  EXH_CUDA_TRY(launch_r2c_rows(RealPairLoad{grid_dev, nd}, HalfStore{work, p->nc}, *p, rows, st));
  EXH_CUDA_TRY(launch_strided(CplxLoad{work, nd, p->nc}, CplxStore{work, nd, p->nc}, p->py, p->twy, -1.f, nd,
                              p->nc, st));
  // x pass + binning
  BinParams bp;
  bp.Nk = Nk;
  bp.kn = (float)(2 * M_PI / L);                      // powermodule.c:7
  bp.kmin = kmin;
  bp.dk = (kmax - kmin) / (float)Nk;                  // powermodule.c:11
  bp.Lb = L / (float)nd;
  bp.Normk = (float)pow((double)(L / (float)(nd * nd)), 1.5);   // spectrum_h.c:90
  bp.window = window;
  const int inner = nd * p->nc;
  // partial histograms: room for the smaller tile width of the two kernels
  const int cap = (int)exh_div_up(inner, 4);
  EXH_TRY(c.buf[B_SCRATCH].ensure((sizeof(double) * 2 + sizeof(unsigned)) * (size_t)cap * Nk));
  double* partP = c.buf[B_SCRATCH].as<double>();
  double* partK = partP + (size_t)cap * Nk;
  unsigned* partN = reinterpret_cast<unsigned*>(partK + (size_t)cap * Nk);
  int nblk = 0;
  {
    KTimer kt(KC_BIN, st, 8.0 * nd * inner);
    EXH_CUDA_TRY(launch_fs_x_bin(work, p->twx, nd, p->nc, bp, partP, partK, partN, cap, &nblk, st));
    if (nblk == 0) {
      nblk = (int)exh_div_up(inner, FFT_W);
      const size_t sm = smem_strided(nd) + (size_t)Nk * (2 * sizeof(double) + sizeof(unsigned)) + 16;
      EXH_CUDA_TRY(set_smem(k_fft_x_bin, sm));
      k_fft_x_bin<<<nblk, FFT_THREADS, sm, st>>>(work, p->px, p->twx, nd, p->nc, bp, partP, partK, partN);
      EXH_CUDA_TRY(cudaGetLastError());
    }
  }
  count_launch(1);
  k_bin_reduce<<<Nk, 256, 0, st>>>(partP, partK, partN, nblk, Nk, outP_dev, outK_dev, outN_dev);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

// ------------------------------------------------------------------------
// Power spectrum that allocates nothing.
//
// Some callers cannot call cudaMalloc: real-time loops that must not stall
// in the allocator (cudaMalloc/cudaFree can synchronise the device), and
// hosts whose device memory is handed out by a pool the caller does not own.  exh_power_compute_noalloc gives them the power
// spectrum of a small grid (nd <= 64, Nk <= 256) with every temporary -- the
// half-complex work array, the twiddle tables and the per-block histograms --
// in one file-scope device array below.  Every GPU that loads the library
// holds that array (about 1.8 MB) until the process exits.  All calls on a
// device share it and it keeps the last call's contents: each call rewrites
// what it reads, and two calls that overlap on the GPU (different streams,
// or different host threads) race on it.
namespace {

constexpr int NA_MAX_ND = 64;
constexpr int NA_MAX_NK = 256;
constexpr int NA_MAX_NC = NA_MAX_ND / 2 + 1;
constexpr int NA_MAX_BLK = (NA_MAX_ND * NA_MAX_NC + FFT_W - 1) / FFT_W;

struct NoAllocScratch {
  float2 work[(size_t)NA_MAX_ND * NA_MAX_ND * NA_MAX_NC];
  float2 twx[NA_MAX_ND], twm[NA_MAX_ND / 2], twn[NA_MAX_ND];
  double partP[NA_MAX_BLK * NA_MAX_NK], partK[NA_MAX_BLK * NA_MAX_NK];
  unsigned partN[NA_MAX_BLK * NA_MAX_NK];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// device address of the array, looked up once per device (with that device
// current); the host-side symbol is only a stand-in and is never passed to
// a kernel
std::mutex g_na_mu;
void* g_na_addr[64] = {};

int noalloc_scratch(int dev, NoAllocScratch** out) {
  if (dev < 0 || dev >= 64) return EXH_E_INVALID;
  std::lock_guard<std::mutex> g(g_na_mu);
  if (!g_na_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      exh_set_error_msg(cudaGetErrorString(e), __FILE__, __LINE__);
      return EXH_E_CUDA;
    }
    g_na_addr[dev] = p;
  }
  *out = reinterpret_cast<NoAllocScratch*>(g_na_addr[dev]);
  return EXH_OK;
}

__global__ void k_na_twiddles(float2* __restrict__ tw, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  double s, c;
  sincospi(2.0 * (double)m / (double)n, &s, &c);
  tw[m] = make_float2((float)c, (float)s);
}

__global__ void k_na_reduce(const double* __restrict__ partP, const double* __restrict__ partK,
                            const unsigned* __restrict__ partN, int nblk, int Nk, float* __restrict__ P,
                            float* __restrict__ K, long long* __restrict__ N) {
  const int b = blockIdx.x;
  __shared__ double rP[128], rK[128];
  __shared__ unsigned long long rN[128];
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
    const unsigned long long n = rN[0];
    N[b] = (long long)n;
    P[b] = n ? (float)(rP[0] / (double)n) : 0.f;
    K[b] = n ? (float)(rK[0] / (double)n) : 0.f;
  }
}

}  // namespace

}  // namespace exh

extern "C" int exh_power_compute_noalloc(const float* grid, int nd, float L, int window, int Nk, float k_min,
                                         float k_max, float* k_out, float* P_out, int64_t* count_out, void* stream) {
  using namespace exh;
  if (!grid || !k_out || !P_out || !count_out) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (nd < 4 || nd > NA_MAX_ND || (nd % 2) != 0 || make_radix_plan(nd).nst < 0 || make_radix_plan(nd / 2).nst < 0) {
    exh_set_error_msg("exh_power_compute_noalloc: nd must be even, 2^a 3^b and at most 64", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (Nk < 1 || Nk > NA_MAX_NK) {
    exh_set_error_msg("exh_power_compute_noalloc: Nk must be in [1, 256]", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (!(L > 0.f) || !(k_max > k_min)) {
    exh_set_error_msg("need L > 0 and k_max > k_min", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (window < 0 || window > 2) {     // as exh_power_compute
    exh_set_error_msg("windows 0 (none), 1 (NGP), 2 (CIC) are built", __FILE__, __LINE__);
    return EXH_E_UNSUPPORTED;
  }
  if (timing_on()) {
    // kernel-class timing creates CUDA events, which this entry point must not
    exh_set_error_msg("exh_power_compute_noalloc: turn kernel-class timing off first", __FILE__, __LINE__);
    return EXH_E_UNSUPPORTED;
  }
  int dev = 0;
  EXH_CUDA_TRY(cudaGetDevice(&dev));
  NoAllocScratch* s = nullptr;
  EXH_TRY(noalloc_scratch(dev, &s));
  cudaStream_t st = (cudaStream_t)stream;
  FFTPlan3D p;
  p.nx = p.ny = p.nz = nd;
  p.nc = nd / 2 + 1;
  p.M = nd / 2;
  p.px = p.py = make_radix_plan(nd);
  p.pm = make_radix_plan(p.M);
  p.twx = p.twy = s->twx;
  p.twm = s->twm;
  p.twn = s->twn;
  k_na_twiddles<<<1, 64, 0, st>>>(s->twx, nd);
  k_na_twiddles<<<1, 64, 0, st>>>(s->twm, p.M);
  k_na_twiddles<<<1, 64, 0, st>>>(s->twn, nd);
  count_launch(3);
  EXH_CUDA_TRY(cudaGetLastError());
  float2* work = s->work;
  const size_t rows = (size_t)nd * nd;
  EXH_CUDA_TRY(launch_r2c_rows(RealPairLoad{grid, nd}, HalfStore{work, p.nc}, p, rows, st));
  EXH_CUDA_TRY(launch_strided(CplxLoad{work, nd, p.nc}, CplxStore{work, nd, p.nc}, p.py, p.twy, -1.f, nd, p.nc, st));
  BinParams bp;
  bp.Nk = Nk;
  bp.kn = (float)(2 * M_PI / L);
  bp.kmin = k_min;
  bp.dk = (k_max - k_min) / (float)Nk;
  bp.Lb = L / (float)nd;
  bp.Normk = (float)pow((double)(L / (float)(nd * nd)), 1.5);
  bp.window = window;
  const int inner = nd * p.nc;
  const int nblk = (int)exh_div_up(inner, FFT_W);
  const size_t sm = smem_strided(nd) + (size_t)Nk * (2 * sizeof(double) + sizeof(unsigned)) + 16;
  EXH_CUDA_TRY(set_smem(k_fft_x_bin, sm));
  k_fft_x_bin<<<nblk, FFT_THREADS, sm, st>>>(work, p.px, p.twx, nd, p.nc, bp, s->partP, s->partK, s->partN);
  k_na_reduce<<<Nk, 128, 0, st>>>(s->partP, s->partK, s->partN, nblk, Nk, P_out, k_out,
                                  reinterpret_cast<long long*>(count_out));
  count_launch(2);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}
