// Galaxy population of a halo catalogue, populate_halos (src/hod/hod.c:31-160)
// -> Populate_total (src/hod/populate_halos.c:120-217), and the colour split,
// split_galaxies (hod.c:163-211) -> Galaxy_Types (split_galaxies.c:37-72).
//
// The reference draws everything from one gsl_rng_taus stream in halo order:
// per halo one uniform for the central (Ncentral_tot >= u), the Poisson draw
// of the satellite number, then (phi, theta, eps) per satellite.  The stream
// is reproduced position for position:
//   1. k_hod_prep      per halo: concentration (f_c or given), <Ncen>, <Nsat>,
//                      concentration range, and whether the satellite draw is
//                      random (<Nsat> > 0: its uniform count depends on the draw)
//   2. k_taus_stream   the stream itself, 64 values per thread from a jump-ahead
//   3. k_hod_parse     one block walks the halos with <Nsat> > 0 in order and
//                      fixes each one's satellite count; a halo with <Nsat> = 0
//                      always takes two uniforms, so only the random ones need
//                      the walk.  Each round draws the next 64 halos at 64
//                      candidate stream offsets in parallel and then follows
//                      the chain of true offsets through shared memory.
//   4. scans           stream offset of every halo (2 i + extra uniforms before
//                      it), galaxies per halo, galaxy offsets
//   5. k_hod_write     central and satellites of every halo, in the reference's
//                      output order, float arithmetic as populate_halos.c
// The r(Eps) splines are built on the host (Interpolate_r_Eps, :56-104) for
// the concentration bins the reference's bin index can reach: that index is
// floor((log c - log cmin) / (log cmax - log cmin)) (:171), 0 for every halo
// but the most concentrated one (1), so bins 0, 1 and 2 are the only ones read.
// The satellite offset is the spline value r itself: R_v is computed at :185
// and not used, as in the reference.
//
// Satellite numbers: gsl_ran_poisson uses Knuth's multiplicative method for
// means up to 10 (k + 1 uniforms for a result k), restated here.  Above 10 GSL
// reduces through gamma and binomial variates; here the multiplicative
// method continues in pieces of mean <= 500, so the stream after a halo with
// more than 10 expected satellites is not GSL's.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "scan.cuh"
#include "setup.h"
#include "taus.cuh"

namespace exh {
namespace {

constexpr double HOD_R_MIN = 1.0e-3;    // hod_h.h:29-35
constexpr double HOD_R_MAX = 10.0;
constexpr int HOD_NRS = 500;
constexpr int HOD_NCS = 100;
constexpr int HOD_NEPS = 1000;
constexpr double HOD_TOL = 0.001;
constexpr int HOD_NB = 3;               // concentration bins the bin index reaches
constexpr int HOD_NEWTON_CAP = 100000;
constexpr double HOD_MU_MAX = 1.0e6;    // largest accepted mean satellite number
constexpr int STREAM_CHUNK = 64;        // stream values per thread
constexpr int HOD_T = 256;

struct HodConst {
  double M0, M1;       // 10^logM0, 10^logM1 (host pow, as the reference)
  double fc_pre;       // 9 / (1 + z) of f_c (:24)
  float Mstar;         // cosmo.Mstar (hod.c:80)
  float logMmin, siglogM, alpha;
  int in_c;
};

struct HodCtl {
  unsigned cmin_bits, cmax_bits;
  int bad_mass, bad_conc, bad_mu;
  int overflow;              // the parse needed stream values beyond the buffer
  double mu_sum;
};

// Ncentral_tot (populate_halos.c:4-6)
__device__ __forceinline__ float ncentral_tot(float M, const HodConst& h) {
  const double a = __ddiv_rn(__dsub_rn(log10((double)M), (double)h.logMmin), (double)h.siglogM);
  return (float)__dmul_rn(0.5, __dadd_rn(1.0, erf(a)));
}

__global__ void __launch_bounds__(HOD_T)
k_hod_prep(const float* __restrict__ Mh, const float* __restrict__ Ch_in, int64_t nh, HodConst h,
           float* __restrict__ Cv, float* __restrict__ pc, float* __restrict__ mu, int* __restrict__ rnd,
           HodCtl* __restrict__ ctl) {
  unsigned lo = 0xFFFFFFFFu, hi = 0u;
  int bm = 0, bc = 0, bu = 0;
  double msum = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x) {
    const float M = Mh[i];
    if (!(M > 0.f) || !isfinite(M)) bm = 1;
    float c;
    if (h.in_c) {
      c = Ch_in[i];
    } else {      // f_c (:21-27): 9/(1+z) (M/Mstar)^-0.13, M/Mstar in float
      c = (float)__dmul_rn(h.fc_pre, pow((double)__fdiv_rn(M, h.Mstar), -0.13));
    }
    if (!(c > 0.f) || !isfinite(c)) bc = 1;
    const float p = ncentral_tot(M, h);
    float m = 0.f;     // Nsatellite_tot (:9-18)
    if ((double)M >= h.M0)
      m = (float)__dmul_rn(pow(__ddiv_rn(__dsub_rn((double)M, h.M0), h.M1), (double)h.alpha), (double)p);
    if (!(m <= (float)HOD_MU_MAX) && !isnan(m)) bu = 1;
    Cv[i] = c;
    pc[i] = p;
    mu[i] = m;
    rnd[i] = m > 0.f ? 1 : 0;      // NaN and 0 draw one uniform, result 0
    lo = min(lo, __float_as_uint(c));
    hi = max(hi, __float_as_uint(c));
    if (m > 0.f) msum += (double)m;
  }
  // positive floats order as their bit patterns
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    msum += __shfl_xor_sync(0xffffffffu, msum, o);
    bm |= __shfl_xor_sync(0xffffffffu, bm, o);
    bc |= __shfl_xor_sync(0xffffffffu, bc, o);
    bu |= __shfl_xor_sync(0xffffffffu, bu, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&ctl->cmin_bits, lo);
    atomicMax(&ctl->cmax_bits, hi);
    if (msum > 0.0) atomicAdd(&ctl->mu_sum, msum);
    if (bm) atomicOr(&ctl->bad_mass, 1);
    if (bc) atomicOr(&ctl->bad_conc, 1);
    if (bu) atomicOr(&ctl->bad_mu, 1);
  }
}

// one halo whose satellite draw is random: the multiplicative draw stops
// at the first uniform u = x / 2^32 with u <= exp(-mu), i.e. x <= thr
struct __align__(8) HodDraw {
  int h;
  unsigned thr;        // floor(exp(-mu) 2^32)
  double emu;          // exp(-mu)
  float emuf;          // exp(-mu) rounded to float
  int mode;            // 0: float test with a certified band, 1: double products, 2: pieces (mu > 500)
};

__global__ void k_hod_compact(const int* __restrict__ rnd, const int* __restrict__ pos, const float* __restrict__ mu,
                              int64_t nh, HodDraw* __restrict__ hm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x)
    if (rnd[i]) {
      const double m = (double)mu[i];
      HodDraw d;
      d.h = (int)i;
      if (m <= 500.0) {
        d.emu = exp(-m);
        d.thr = (unsigned)floor(__dmul_rn(d.emu, 4294967296.0));   // exact scaling; emu < 1
        d.emuf = (float)d.emu;
        d.mode = m <= 60.0 ? 0 : 1;            // exp(-60) ~ 1e-26 stays a normal float
      } else {
        d.emu = 0.0;
        d.thr = 0u;
        d.emuf = 0.f;
        d.mode = 2;
      }
      hm[pos[i]] = d;
    }
}

// stream values [t*CHUNK, (t+1)*CHUNK): value p is the (p+1)-th draw after seeding
__global__ void __launch_bounds__(128)
k_taus_stream(const TausJump* __restrict__ J, TausState s0, unsigned* __restrict__ out, int64_t n) {
  const int64_t p0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * STREAM_CHUNK;
  if (p0 >= n) return;
  unsigned s[3] = {s0.s[0], s0.s[1], s0.s[2]};
  taus_jump(J, s, (unsigned long long)p0);
  uint4* o4 = reinterpret_cast<uint4*>(out + p0);
#pragma unroll 4
  for (int q = 0; q < STREAM_CHUNK / 4; q++) {
    uint4 v;
    v.x = taus_next(s);
    v.y = taus_next(s);
    v.z = taus_next(s);
    v.w = taus_next(s);
    o4[q] = v;            // n is a multiple of STREAM_CHUNK
  }
}

// gsl_ran_poisson's multiplicative branch from stream position p; pieces of
// mean <= 500 above it.  Returns false when the stream ends first.
__device__ __forceinline__ bool hod_poisson(double mu, const unsigned* __restrict__ st, int64_t Ls, int64_t p,
                                            int* k_out, int* used_out) {
  int total = 0, used = 0;
  double rem = mu;
  for (;;) {
    const double m = rem > 500.0 ? 500.0 : rem;
    const double emu = exp(-m);
    double prod = 1.0;
    int k = 0;
    do {
      if (p + used >= Ls) return false;
      prod = __dmul_rn(prod, taus_u01(st[p + used]));
      used++;
      k++;
    } while (prod > emu);
    total += k - 1;
    rem = __dsub_rn(rem, m);
    if (!(rem > 0.0)) break;
  }
  *k_out = total;
  *used_out = used;
  return true;
}

// Satellite counts of the halos with a random draw, in halo order, by one
// block.  A round takes the next PARSE_H halos and draws each of them at
// PARSE_C candidate offsets E, E+4, ..., E+4(PARSE_C-1) (E: uniforms beyond
// two per halo so far; a halo with ns satellites from the multiplicative
// draw takes 4 ns more, so E moves in steps of 4).  Thread 0 then follows
// the chain through shared memory: halo q reads its result at the offset
// the halos before it left, while that offset is a candidate.  At least one
// halo commits per round (the first one's candidate 0 is exact).
constexpr int PARSE_H = 64;
constexpr int PARSE_C = 64;
constexpr int PARSE_T = 512;
constexpr int PARSE_HPW = PARSE_H / (PARSE_T / 32);       // halos per warp
constexpr int PARSE_PER = PARSE_H * PARSE_C / PARSE_T;    // candidates per thread

constexpr int PARSE_PRE = 3;     // stream values fetched ahead per candidate

// the double product u_p u_{p+1} ... u_{p+n-1} in the draw's order
__device__ __noinline__ double hod_prod(const unsigned* __restrict__ st, int64_t p, int n) {
  double pr = taus_u01(st[p]);
  for (int j = 1; j < n; j++) pr = __dmul_rn(pr, taus_u01(st[p + j]));
  return pr;
}

// stream value p + u: from the prefetched ones when u < PARSE_PRE
__device__ __forceinline__ unsigned hod_value(const unsigned (&x)[PARSE_PRE], const unsigned* __restrict__ st,
                                              int64_t p, int u) {
  unsigned v = 0u;
  bool hit = false;
#pragma unroll
  for (int j = 1; j < PARSE_PRE; j++)
    if (u == j) { v = x[j]; hit = true; }
  return hit ? v : st[p + u];
}

// The draw of one halo from stream position p; x[] holds the values at
// p .. p + PARSE_PRE - 1 (those below Ls).  The multiplicative draw goes on
// while the double product exceeds exp(-mu).  In mode 0 the product is
// carried in float: after n factors its relative distance to the double
// product is below n 2^-23 (n roundings of the factors and n - 1 of the
// products, each 2^-24) and exp(-mu) in float is within 2^-24, so a float
// product outside emuf (1 +- (n + 3) 2^-22) decides the comparison; inside
// that band the double product is formed and compared as the reference does.
__device__ __forceinline__ bool hod_draw(const HodDraw& d, const unsigned (&x)[PARSE_PRE],
                                         const float* __restrict__ mu, const unsigned* __restrict__ st, int64_t Ls,
                                         int64_t p, int* ns, int* used) {
  if (d.mode == 2) return hod_poisson((double)mu[d.h], st, Ls, p, ns, used);
  if (p >= Ls) return false;
  if (x[0] <= d.thr) { *ns = 0; *used = 1; return true; }
  constexpr float TWO_M32 = 2.3283064365386963e-10f;
  constexpr float TWO_M22 = 2.384185791015625e-07f;
  if (d.mode == 0) {
    float pf = __fmul_rn((float)x[0], TWO_M32);
    int u = 1;
    for (;;) {
      if (p + u >= Ls) return false;
      const unsigned v = hod_value(x, st, p, u);
      pf = __fmul_rn(pf, __fmul_rn((float)v, TWO_M32));
      u++;
      const float tol = __fmul_rn((float)(u + 3), TWO_M22);
      bool more;
      if (pf > __fmul_rn(d.emuf, __fadd_rn(1.f, tol))) more = true;
      else if (pf < __fmul_rn(d.emuf, __fsub_rn(1.f, tol))) more = false;
      else more = hod_prod(st, p, u) > d.emu;
      if (!more) break;
    }
    *ns = u - 1;
    *used = u;
    return true;
  }
  double prod = taus_u01(x[0]);
  int u = 1;
  do {
    if (p + u >= Ls) return false;
    const unsigned v = hod_value(x, st, p, u);
    prod = __dmul_rn(prod, taus_u01(v));
    u++;
  } while (prod > d.emu);
  *ns = u - 1;
  *used = u;
  return true;
}

__global__ void __launch_bounds__(PARSE_T)
k_hod_parse(const HodDraw* __restrict__ hm, int K, const float* __restrict__ mu, const unsigned* __restrict__ st,
            int64_t Ls, int* __restrict__ nsat, long long* __restrict__ extra, HodCtl* __restrict__ ctl) {
  __shared__ int s_ns[PARSE_H][PARSE_C];     // [halo][candidate]: a warp writes consecutive words
  __shared__ int s_ex[PARSE_H][PARSE_C];      // -1: stream ended first
  __shared__ unsigned long long s_Z[PARSE_C];  // bit q: halo q moves the offset (or ran out) at candidate c
  __shared__ int s_cs[PARSE_H];                 // candidate of the run starting at halo q
  __shared__ unsigned long long s_B;            // bit q: a run starts at halo q
  __shared__ long long s_E;
  __shared__ int s_k, s_adv, s_ovf;
  if (threadIdx.x == 0) { s_E = 0; s_k = 0; s_ovf = 0; s_adv = 0; }
  if (threadIdx.x < PARSE_C) s_Z[threadIdx.x] = 0ull;
  __syncthreads();
  // warp w: halos PARSE_HPW w .. + PARSE_HPW - 1 of the round; lane l:
  // candidates l and l + 32, so a warp's loads cover one halo's consecutive
  // candidate offsets
  const int lane = threadIdx.x & 31, wq = (threadIdx.x >> 5) * PARSE_HPW;
  static_assert(PARSE_PER == 2 * PARSE_HPW && PARSE_C == 64, "round shape");
  for (;;) {
    const int k = s_k;
    const long long E = s_E;
    if (k >= K) break;
    HodDraw d[PARSE_HPW];
    bool valid[PARSE_HPW];
#pragma unroll
    for (int a = 0; a < PARSE_HPW; a++) {
      valid[a] = k + wq + a < K;
      d[a] = valid[a] ? hm[k + wq + a] : HodDraw{0, 0u, 0.0, 0.f, 0};
    }
    unsigned x[PARSE_PER][PARSE_PRE];
#pragma unroll
    for (int i = 0; i < PARSE_PER; i++) {
      const int a = i >> 1, c = lane + 32 * (i & 1);
      const int64_t pp = 2 * (int64_t)d[a].h + E + 4 * c + 1;
#pragma unroll
      for (int j = 0; j < PARSE_PRE; j++) x[i][j] = valid[a] && pp + j < Ls ? st[pp + j] : 0u;
    }
#pragma unroll
    for (int i = 0; i < PARSE_PER; i++) {
      const int a = i >> 1, c = lane + 32 * (i & 1);
      const int64_t pp = 2 * (int64_t)d[a].h + E + 4 * c + 1;
      int ns = 0, used = 0, ex = -1;
      if (valid[a] && hod_draw(d[a], x[i], mu, st, Ls, pp, &ns, &used)) ex = used + 3 * ns - 1;
      s_ns[wq + a][c] = ns;
      s_ex[wq + a][c] = ex;
      if (ex != 0) atomicOr(&s_Z[c], 1ull << (wq + a));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      // follow the offsets from candidate 0, jumping over the halos that
      // leave the offset where it is
      const int lim = min(PARSE_H, K - k);
      const unsigned long long live = lim >= 64 ? ~0ull : ((1ull << lim) - 1ull);
      int c = 0, adv = lim, rel = 0;
      unsigned long long B = 1ull, from = live;      // halos not yet passed
      s_cs[0] = 0;
      for (;;) {
        const unsigned long long z = s_Z[c] & from;
        if (z == 0ull) { rel = 4 * c; break; }
        const int qq = __ffsll((long long)z) - 1;
        const int ex = s_ex[qq][c];
        if (ex < 0) { s_ovf = 1; break; }
        rel = 4 * c + ex;
        if (qq + 1 >= lim || (rel & 3) || rel >= 4 * PARSE_C) { adv = qq + 1; break; }
        c = rel >> 2;
        from = live & (~1ull << qq);                  // halos qq + 1 ..
        B |= 1ull << (qq + 1);
        s_cs[qq + 1] = c;
      }
      s_B = B;
      s_adv = adv;
      s_E = E + rel;
      s_k = k + adv;
    }
    __syncthreads();
    if (s_ovf) {
      if (threadIdx.x == 0) ctl->overflow = 1;
      return;
    }
    if (threadIdx.x < s_adv) {
      const int qq = threadIdx.x;
      const unsigned long long upto = qq == 63 ? ~0ull : ((2ull << qq) - 1ull);
      const int c = s_cs[63 - __clzll((long long)(s_B & upto))];    // the run holding halo qq
      const int h = hm[k + qq].h;
      nsat[h] = s_ns[qq][c];
      extra[h] = s_ex[qq][c];
    }
    if (threadIdx.x < PARSE_C) s_Z[threadIdx.x] = 0ull;
    __syncthreads();
  }
}

// galaxies per halo: the central draw at offset 2 i + E_i
__global__ void __launch_bounds__(HOD_T)
k_hod_count(const float* __restrict__ pc, const int* __restrict__ nsat, const long long* __restrict__ E,
            const unsigned* __restrict__ st, int64_t nh, long long* __restrict__ ngal) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nh; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = 2 * i + E[i];
    const int cen = (double)pc[i] >= taus_u01(st[o]) ? 1 : 0;
    ngal[i] = cen + nsat[i];
  }
}

struct HodWriteArgs {
  const float* posh;
  const float* velh;
  const float* Cv;
  const int* nsat;
  const long long* extra;   // uniforms beyond two of each halo
  const long long* E;       // exclusive sum of extra
  const long long* G;       // first galaxy of each halo
  const long long* ngal;
  const unsigned* st;
  DevSpline r[HOD_NB];
  double cb[HOD_NB];        // bin concentrations pow(10, log cmin + (log cmax - log cmin) k / 99)
  float cmin, cmax;
  float L[3];
  int64_t nh;
  float* posg;
  float* velg;
  long long* flag;
  int* err;
};

// cysumf (hod_h.c:4-13)
__device__ __forceinline__ float hod_wrap(float x, float y, float L) {
  float r = __fadd_rn(x, y);
  if (r >= L) r = __fsub_rn(r, L);
  if (r < 0.f) r = __fadd_rn(r, L);
  return r;
}

__global__ void __launch_bounds__(HOD_T) k_hod_write(HodWriteArgs a) {
  int bad = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.nh; i += (int64_t)gridDim.x * blockDim.x) {
    const long long n = a.ngal[i];
    if (n == 0) continue;
    const int ns = a.nsat[i];
    long long g = a.G[i];
    const int64_t o = 2 * i + a.E[i];
    const float px = a.posh[3 * i], py = a.posh[3 * i + 1], pz = a.posh[3 * i + 2];
    float vx = 0.f, vy = 0.f, vz = 0.f;
    if (a.velg) { vx = a.velh[3 * i]; vy = a.velh[3 * i + 1]; vz = a.velh[3 * i + 2]; }
    if (n > ns) {           // the central (:149-160)
      a.posg[3 * g] = px; a.posg[3 * g + 1] = py; a.posg[3 * g + 2] = pz;
      if (a.velg) { a.velg[3 * g] = vx; a.velg[3 * g + 1] = vy; a.velg[3 * g + 2] = vz; }
      a.flag[g] = -(long long)i;
      g++;
    }
    if (ns == 0) continue;
    // bin index and weights (:170-178)
    int ind = 0;
    float w1, w2;
    const float C = a.Cv[i];
    if (a.cmax == a.cmin) {       // the reference divides 0 by 0 here
      w1 = 0.f;
      w2 = 1.f;
    } else {
      const double lc0 = log10((double)a.cmin);
      const double f = floor(__ddiv_rn(__dsub_rn(log10((double)C), lc0), __dsub_rn(log10((double)a.cmax), lc0)));
      ind = f >= 1.0 ? 1 : 0;
      w1 = (float)__dsub_rn((double)C, a.cb[ind]);
      w2 = (float)__dsub_rn(a.cb[ind + 1], (double)C);
      const float Rv = __fadd_rn(w1, w2);
      w1 = __fdiv_rn(w1, Rv);
      w2 = __fdiv_rn(w2, Rv);
    }
    // (phi, theta, eps) of each satellite follow the central and Poisson draws
    const long long used = a.extra[i] - 3LL * ns + 1;
    const int64_t p = o + 1 + used;
    for (int j = 0; j < ns; j++, g++) {
      const int64_t q = p + 3 * (int64_t)j;
      const float phi = (float)__dmul_rn(6.283185307179586, taus_u01(a.st[q]));
      const float theta = (float)__dmul_rn(3.14159265358979323846, taus_u01(a.st[q + 1]));
      const double eps = (double)(float)taus_u01(a.st[q + 2]);
      const float r1 = (float)a.r[ind].eval(eps, &bad);          // Generate_r (:107-117)
      const float r2 = (float)a.r[ind + 1].eval(eps, &bad);
      const float r = __fadd_rn(__fmul_rn(r1, w1), __fmul_rn(r2, w2));
      const double rs = __dmul_rn((double)r, sin((double)theta));
      a.posg[3 * g] = hod_wrap(px, (float)__dmul_rn(rs, cos((double)phi)), a.L[0]);
      a.posg[3 * g + 1] = hod_wrap(py, (float)__dmul_rn(rs, sin((double)phi)), a.L[1]);
      a.posg[3 * g + 2] = hod_wrap(pz, (float)__dmul_rn((double)r, cos((double)theta)), a.L[2]);
      if (a.velg) { a.velg[3 * g] = vx; a.velg[3 * g + 1] = vy; a.velg[3 * g + 2] = vz; }
      a.flag[g] = (long long)i;
    }
  }
  if (bad) atomicExch(a.err, 1);
}

// Galaxy_Types (split_galaxies.c:37-72): one uniform per galaxy, in order
constexpr int SPLIT_CHUNK = 8;

__global__ void __launch_bounds__(128)
k_hod_split(const TausJump* __restrict__ J, TausState s0, const float* __restrict__ Mh, int64_t nh,
            const long long* __restrict__ flag, int64_t ng, const float* __restrict__ pcen,
            const float* __restrict__ psat, int ntypes, int order_cen, int order_sat, int* __restrict__ type,
            int* __restrict__ err) {
  const int64_t g0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * SPLIT_CHUNK;
  if (g0 >= ng) return;
  unsigned s[3] = {s0.s[0], s0.s[1], s0.s[2]};
  taus_jump(J, s, (unsigned long long)g0);
  const int64_t g1 = min(ng, g0 + SPLIT_CHUNK);
  int bad = 0;
  for (int64_t g = g0; g < g1; g++) {
    const float rnd = (float)taus_u01(taus_next(s));
    const long long f = flag[g];
    const long long hh = f > 0 ? f : -f;
    if (hh >= nh || hh < 0) { bad = 1; type[g] = 0; continue; }
    const float lm = (float)log10((double)Mh[hh]);
    const bool sat = f > 0;
    const float* P = sat ? psat : pcen;
    const int order = sat ? order_sat : order_cen;
    float occ = 0.f;
    int t = 0;
    for (int j = 0; j < ntypes - 1; j++) {
      float resp = 0.f;              // Occ_cen / Occ_sat (:4-33)
      for (int q = 0; q < order; q++)
        resp = (float)__dadd_rn((double)resp, __dmul_rn((double)P[j * order + q], pow((double)lm, (double)q)));
      if (resp < 0.f) resp = 0.f;
      if (resp > 1.f) resp = 1.f;
      occ = __fadd_rn(occ, resp);
      if (rnd <= occ) { t = j + 1; break; }
    }
    if (rnd > occ) t = ntypes;
    type[g] = sat ? t : -t;
  }
  if (bad) atomicExch(err, 1);
}

// ---------------------------------------------------------------- host
// Profile (populate_halos.c:30-36) in the reference's float/double mix
float hod_profile(float x, float c, float sigma) {
  const float cx = c * x;
  return (float)(1.0 / ((double)cx * std::pow(1.0 + (double)cx, 2.0)) / (1.0 + std::pow((double)x, 2.0 / (double)sigma)));
}

double hod_bin_conc(float cmin, float cmax, int k) {
  return std::pow(10.0, std::log10((double)cmin) + (std::log10((double)cmax) - std::log10((double)cmin)) * k /
                            (HOD_NCS - 1));
}

// Interpolate_r_Eps (:56-104) for concentration bin k: r(Eps) knots
int hod_r_table(float cmin, float cmax, int k, float sigma, std::vector<double>& r) {
  std::vector<double> x(HOD_NRS), Int(HOD_NRS);
  for (int i = 0; i < HOD_NRS; i++)
    x[i] = std::pow(10.0, std::log10(HOD_R_MIN) + (std::log10(HOD_R_MAX) - std::log10(HOD_R_MIN)) * i /
                              (HOD_NRS - 1));
  const float c = (float)hod_bin_conc(cmin, cmax, k);
  Int[0] = 0.0;
  for (int j = 1; j < HOD_NRS; j++)
    Int[j] = Int[j - 1] + ((double)hod_profile((float)x[j], c, sigma) * x[j] * x[j] +
                           (double)hod_profile((float)x[j - 1], c, sigma) * x[j - 1] * x[j - 1]) *
                              (x[j] - x[j - 1]) / 2.0;
  Spline sI;
  if (sI.init(x.data(), Int.data(), HOD_NRS) != EXH_OK) return EXH_E_RANGE;
  int bad = 0;
  const float A = (float)sI.eval(HOD_R_MAX, &bad);
  r.assign(HOD_NEPS, 0.0);
  r[0] = HOD_R_MIN;
  for (int j = 1; j < HOD_NEPS - 1 && !bad; j++) {
    const double eps = ((double)j) / (HOD_NEPS - 1);
    r[j] = j > 1 ? r[j - 1] : HOD_R_MIN + eps;
    float rtmp = (float)(r[j] + 1.0);
    int it = 0;
    while (std::fabs(r[j] - (double)rtmp) > HOD_TOL) {
      if (++it > HOD_NEWTON_CAP) { bad = 1; break; }
      rtmp = (float)r[j];
      r[j] = r[j] - (sI.eval(r[j], &bad) / (double)A - eps) /
                        ((double)hod_profile((float)r[j], c, sigma) * r[j] * r[j] / (double)A);
      if (r[j] >= HOD_R_MAX || r[j] <= HOD_R_MIN) r[j] = eps;
    }
  }
  r[HOD_NEPS - 1] = HOD_R_MAX;
  return bad ? EXH_E_RANGE : EXH_OK;
}

// bump allocation inside one device buffer, 256-byte aligned pieces
struct Bump {
  char* base;
  size_t off = 0;
  template <class T> T* take(size_t n) {
    T* p = reinterpret_cast<T*>(base + off);
    off += (sizeof(T) * n + 255) & ~size_t(255);
    return p;
  }
};

}  // namespace
}  // namespace exh

using namespace exh;

extern "C" int exh_hod_populate(exh_ctx* ctx, const float* posh, const float* velh, const float* Mh, const float* Ch,
                                int64_t nh, const exh_hod_params* hp, int out_vel, int64_t* ng_out, int mem,
                                void* stream) {
  if (!ctx || !hp || !ng_out || (nh > 0 && (!posh || !Mh || (out_vel && !velh)))) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (nh < 0 || nh > (int64_t)1 << 30 || !(hp->Lc > 0.f) || !std::isfinite(hp->Lc) || hp->ndx < 0 || hp->ndy < 0 ||
      hp->ndz < 0) {
    exh_set_error_msg("need 0 <= nh <= 2^30, Lc > 0 and non-negative grid sizes", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  c.hod_ng = -1;
  c.hod_vel = out_vel ? 1 : 0;
  *ng_out = 0;
  if (nh == 0) {
    c.hod_ng = 0;
    return EXH_OK;
  }
  const size_t n = (size_t)nh;
  // inputs on the device
  const float *dpos = posh, *dvel = out_vel ? velh : nullptr, *dM = Mh, *dC = Ch;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_HODIN].ensure(sizeof(float) * n * 8 + 1024));
    Bump in{c.buf[B_HODIN].as<char>()};
    float* a = in.take<float>(3 * n);
    EXH_CUDA_TRY(cudaMemcpyAsync(a, posh, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    dpos = a;
    if (out_vel) {
      float* v = in.take<float>(3 * n);
      EXH_CUDA_TRY(cudaMemcpyAsync(v, velh, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
      dvel = v;
    }
    float* m = in.take<float>(n);
    EXH_CUDA_TRY(cudaMemcpyAsync(m, Mh, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    dM = m;
    if (Ch) {
      float* q = in.take<float>(n);
      EXH_CUDA_TRY(cudaMemcpyAsync(q, Ch, sizeof(float) * n, cudaMemcpyHostToDevice, st));
      dC = q;
    }
  }
  // per-halo work
  const size_t nscan = n / SCAN_TILE + 2;
  const size_t work_bytes = n * (4 * 6 + 8 * 4 + sizeof(HodDraw)) + nscan * 16 + sizeof(TausJump) + 8 * HOD_NEPS * (1 + 2 * HOD_NB) +
                            32 * 256;
  EXH_TRY(c.buf[B_HOD].ensure(work_bytes));
  Bump w{c.buf[B_HOD].as<char>()};
  float* Cv = w.take<float>(n);
  float* pc = w.take<float>(n);
  float* mu = w.take<float>(n);
  int* rnd = w.take<int>(n);
  int* rpos = w.take<int>(n);
  HodDraw* hm = w.take<HodDraw>(n);
  int* nsat = w.take<int>(n);
  long long* extra = w.take<long long>(n);
  long long* E = w.take<long long>(n);
  long long* ngal = w.take<long long>(n);
  long long* G = w.take<long long>(n);
  long long* sc = w.take<long long>(nscan);
  int* isc = w.take<int>(nscan);
  HodCtl* ctl = w.take<HodCtl>(1);
  int* K_dev = w.take<int>(1);
  long long* tot = w.take<long long>(2);       // extra total, galaxy total
  int* werr = w.take<int>(1);
  TausJump* dJ = w.take<TausJump>(1);
  double* dtab = w.take<double>((size_t)HOD_NEPS * (1 + 2 * HOD_NB));

  HodConst hc{};
  hc.M0 = std::pow(10.0, (double)hp->logM0);
  hc.M1 = std::pow(10.0, (double)hp->logM1);
  hc.fc_pre = 9.0 / (1.0 + (double)hp->redshift);
  hc.Mstar = 4.638211e+12f;
  hc.logMmin = hp->logMmin;
  hc.siglogM = hp->siglogM;
  hc.alpha = hp->alpha;
  hc.in_c = dC ? 1 : 0;
  const HodCtl ctl0{0xFFFFFFFFu, 0u, 0, 0, 0, 0, 0.0};
  static_assert(sizeof(ctl0) <= UPLOAD_SMALL_MAX, "control block fits a kernel argument");
  EXH_TRY(upload_small(ctl, &ctl0, sizeof(ctl0), st));
  EXH_CUDA_TRY(cudaMemsetAsync(nsat, 0, sizeof(int) * n, st));
  EXH_CUDA_TRY(cudaMemsetAsync(extra, 0, sizeof(long long) * n, st));
  const unsigned nb = (unsigned)std::min<size_t>(exh_div_up(n, HOD_T), EXH_NUM_SMS * 8);
  k_hod_prep<<<nb, HOD_T, 0, st>>>(dM, dC, nh, hc, Cv, pc, mu, rnd, ctl);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  EXH_CUDA_TRY(exclusive_scan<int>(rnd, rpos, n, isc, K_dev, st));
  k_hod_compact<<<nb, HOD_T, 0, st>>>(rnd, rpos, mu, nh, hm);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  HodCtl hctl;
  int K = 0;
  EXH_CUDA_TRY(cudaMemcpyAsync(&hctl, ctl, sizeof(hctl), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaMemcpyAsync(&K, K_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  if (hctl.bad_mass) {
    exh_set_error_msg("halo masses must be finite and positive", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (hctl.bad_conc) {
    exh_set_error_msg("halo concentrations must be finite and positive", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (hctl.bad_mu) {
    exh_set_error_msg("mean satellite number above 1e6 (check logM1 and alpha)", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  float cmin, cmax;
  std::memcpy(&cmin, &hctl.cmin_bits, 4);
  std::memcpy(&cmax, &hctl.cmax_bits, 4);

  // stream: two uniforms per halo plus a generous bound on the extra ones
  const TausJump& J = taus_jump_host();
  TausState s0;
  taus_seed_state((unsigned long)(unsigned)hp->seed, s0.s);
  EXH_CUDA_TRY(cudaMemcpyAsync(dJ, &J, sizeof(J), cudaMemcpyHostToDevice, st));
  const double mus = hctl.mu_sum;
  int64_t Ls = 2 * nh + 4 * (int64_t)std::ceil(mus + 10.0 * std::sqrt(mus) + 64.0) + (int64_t)(mus / 500.0) + K + 4096;
  unsigned* dst = nullptr;
  for (int attempt = 0;; attempt++) {
    Ls = (Ls + STREAM_CHUNK - 1) / STREAM_CHUNK * STREAM_CHUNK;
    if (Ls >= ((int64_t)1 << 32) || attempt > 8) {
      exh_set_error_msg("random stream longer than 2^32 values", __FILE__, __LINE__);
      return EXH_E_RANGE;
    }
    EXH_TRY(c.buf[B_HODG].ensure(sizeof(unsigned) * (size_t)Ls));   // reused for the galaxies below
    dst = c.buf[B_HODG].as<unsigned>();
    k_taus_stream<<<exh_div_up((size_t)(Ls / STREAM_CHUNK), 128), 128, 0, st>>>(dJ, s0, dst, Ls);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
    EXH_CUDA_TRY(cudaMemsetAsync(&ctl->overflow, 0, sizeof(int), st));
    if (K > 0) {
      k_hod_parse<<<1, PARSE_T, 0, st>>>(hm, K, mu, dst, Ls, nsat, extra, ctl);
      count_launch(1);
      EXH_CUDA_TRY(cudaGetLastError());
    }
    EXH_CUDA_TRY(exclusive_scan<long long>(extra, E, n, sc, &tot[0], st));
    int ovf = 0;
    long long etot = 0;
    EXH_CUDA_TRY(cudaMemcpyAsync(&ovf, &ctl->overflow, sizeof(int), cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaMemcpyAsync(&etot, &tot[0], sizeof(long long), cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    if (ovf) { Ls *= 2; continue; }
    if (2 * nh + etot > Ls) { Ls = 2 * nh + etot; continue; }      // the counts stand; regenerate longer
    break;
  }
  // the r(Eps) splines of bins 0..2 while the device is idle
  HodWriteArgs wa{};
  {
    std::vector<double> h(HOD_NEPS * (1 + 2 * HOD_NB));
    for (int i = 0; i < HOD_NEPS; i++) h[i] = ((double)i) / (HOD_NEPS - 1);
    for (int k = 0; k < HOD_NB; k++) {
      std::vector<double> r;
      if (hod_r_table(cmin, cmax, k, hp->sigma, r) != EXH_OK) {
        exh_set_error_msg("r(Eps) table: the profile integral left its spline or Newton did not settle", __FILE__,
                          __LINE__);
        return EXH_E_RANGE;
      }
      Spline sr;
      if (sr.init(h.data(), r.data(), HOD_NEPS) != EXH_OK) return EXH_E_RANGE;
      std::memcpy(&h[HOD_NEPS * (1 + 2 * k)], sr.y.data(), sizeof(double) * HOD_NEPS);
      std::memcpy(&h[HOD_NEPS * (2 + 2 * k)], sr.c.data(), sizeof(double) * HOD_NEPS);
      wa.cb[k] = hod_bin_conc(cmin, cmax, k);
    }
    EXH_CUDA_TRY(cudaMemcpyAsync(dtab, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));    // h dies here
  }
  k_hod_count<<<nb, HOD_T, 0, st>>>(pc, nsat, E, dst, nh, ngal);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  EXH_CUDA_TRY(exclusive_scan<long long>(ngal, G, n, sc, &tot[1], st));
  long long ng = 0;
  EXH_CUDA_TRY(cudaMemcpyAsync(&ng, &tot[1], sizeof(long long), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  // galaxies after the stream in the same buffer
  const size_t soff = ((size_t)Ls * sizeof(unsigned) + 255) & ~size_t(255);
  const size_t gbytes = soff + (size_t)ng * (12 + (out_vel ? 12 : 0) + 8) + 1024;
  if (gbytes > c.buf[B_HODG].cap) {
    // grow: keep the stream by copying it into the grown buffer
    DevBuf nbuf;
    EXH_TRY(nbuf.ensure(gbytes));
    EXH_CUDA_TRY(cudaMemcpyAsync(nbuf.p, dst, sizeof(unsigned) * (size_t)Ls, cudaMemcpyDeviceToDevice, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    c.buf[B_HODG].release();
    c.buf[B_HODG] = nbuf;
    nbuf.p = nullptr;
    dst = c.buf[B_HODG].as<unsigned>();
  }
  Bump gb{c.buf[B_HODG].as<char>(), soff};
  wa.posg = gb.take<float>(3 * (size_t)ng);
  wa.velg = out_vel ? gb.take<float>(3 * (size_t)ng) : nullptr;
  wa.flag = gb.take<long long>((size_t)ng);
  wa.posh = dpos;
  wa.velh = dvel;
  wa.Cv = Cv;
  wa.nsat = nsat;
  wa.extra = extra;
  wa.E = E;
  wa.G = G;
  wa.ngal = ngal;
  wa.st = dst;
  for (int k = 0; k < HOD_NB; k++)
    wa.r[k] = DevSpline{dtab, dtab + HOD_NEPS * (1 + 2 * k), dtab + HOD_NEPS * (2 + 2 * k), HOD_NEPS};
  wa.cmin = cmin;
  wa.cmax = cmax;
  wa.L[0] = hp->Lc * (float)hp->ndx;     // hod_h.c:62-64 (0 when the grid size is 0: no wrap)
  wa.L[1] = hp->Lc * (float)hp->ndy;
  wa.L[2] = hp->Lc * (float)hp->ndz;
  wa.nh = nh;
  wa.err = werr;
  EXH_CUDA_TRY(cudaMemsetAsync(werr, 0, sizeof(int), st));
  k_hod_write<<<nb, HOD_T, 0, st>>>(wa);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  EXH_CUDA_TRY(cudaMemcpyAsync(&herr, werr, sizeof(int), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    exh_set_error_msg("satellite radius outside the r(Eps) table", __FILE__, __LINE__);
    return EXH_E_RANGE;
  }
  c.hod_ng = ng;
  c.hod_off = soff;
  *ng_out = ng;
  return EXH_OK;
}

extern "C" int exh_hod_fetch(exh_ctx* ctx, float* posg, float* velg, int64_t* flag, int mem, void* stream) {
  if (!ctx) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  Ctx& c = ctx->c;
  if (c.hod_ng < 0) {
    exh_set_error_msg("no galaxy catalogue: call exh_hod_populate first", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (velg && !c.hod_vel) {
    exh_set_error_msg("the catalogue was populated without velocities", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  const size_t ng = (size_t)c.hod_ng;
  if (ng == 0) return EXH_OK;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  Bump gb{c.buf[B_HODG].as<char>(), c.hod_off};
  const float* dp = gb.take<float>(3 * ng);
  const float* dv = c.hod_vel ? gb.take<float>(3 * ng) : nullptr;
  const long long* df = gb.take<long long>(ng);
  const cudaMemcpyKind kind = mem == EXH_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (posg) EXH_CUDA_TRY(cudaMemcpyAsync(posg, dp, sizeof(float) * 3 * ng, kind, st));
  if (velg) EXH_CUDA_TRY(cudaMemcpyAsync(velg, dv, sizeof(float) * 3 * ng, kind, st));
  if (flag) EXH_CUDA_TRY(cudaMemcpyAsync(flag, df, sizeof(long long) * ng, kind, st));
  if (mem == EXH_MEM_HOST) EXH_CUDA_TRY(cudaStreamSynchronize(st));
  return EXH_OK;
}

extern "C" int exh_hod_split(exh_ctx* ctx, const float* Mh, int64_t nh, const int64_t* flag, int64_t ng,
                             const float* params_cen, const float* params_sat, int ntypes, int order_cen,
                             int order_sat, int seed, int32_t* type_out, int mem, void* stream) {
  if (!ctx || (ng > 0 && (!Mh || !flag || !type_out || !params_cen || !params_sat))) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (nh < 0 || ng < 0 || ntypes < 2 || order_cen < 1 || order_sat < 1 || order_cen > 64 || order_sat > 64 ||
      ntypes > 4096) {
    exh_set_error_msg("need ntypes >= 2, 1 <= polynomial orders <= 64", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (ng == 0) return EXH_OK;
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t npc = (size_t)(ntypes - 1) * order_cen, nps = (size_t)(ntypes - 1) * order_sat;
  const size_t bytes = sizeof(TausJump) + sizeof(float) * (npc + nps) + sizeof(int) * 64 + 1024 +
                       (mem == EXH_MEM_HOST ? sizeof(float) * (size_t)nh + 12 * (size_t)ng + 1024 : 0);
  EXH_TRY(c.buf[B_HODIN].ensure(bytes));
  Bump w{c.buf[B_HODIN].as<char>()};
  TausJump* dJ = w.take<TausJump>(1);
  float* dpc = w.take<float>(npc);
  float* dps = w.take<float>(nps);
  int* derr = w.take<int>(1);
  const float* dM = Mh;
  const long long* dflag = reinterpret_cast<const long long*>(flag);
  int* dtype = type_out;
  const cudaMemcpyKind pk = mem == EXH_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  EXH_CUDA_TRY(cudaMemcpyAsync(dJ, &taus_jump_host(), sizeof(TausJump), cudaMemcpyHostToDevice, st));
  EXH_CUDA_TRY(cudaMemcpyAsync(dpc, params_cen, sizeof(float) * npc, pk, st));
  EXH_CUDA_TRY(cudaMemcpyAsync(dps, params_sat, sizeof(float) * nps, pk, st));
  if (mem == EXH_MEM_HOST) {
    float* m = w.take<float>((size_t)nh);
    long long* f = w.take<long long>((size_t)ng);
    int* t = w.take<int>((size_t)ng);
    if (nh > 0) EXH_CUDA_TRY(cudaMemcpyAsync(m, Mh, sizeof(float) * (size_t)nh, cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaMemcpyAsync(f, flag, sizeof(long long) * (size_t)ng, cudaMemcpyHostToDevice, st));
    dM = m;
    dflag = f;
    dtype = t;
  }
  EXH_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), st));
  TausState s0;
  taus_seed_state((unsigned long)(unsigned)seed, s0.s);
  k_hod_split<<<exh_div_up(exh_div_up((size_t)ng, SPLIT_CHUNK), 128), 128, 0, st>>>(
      dJ, s0, dM, nh, dflag, ng, dpc, dps, ntypes, order_cen, order_sat, dtype, derr);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  EXH_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (mem == EXH_MEM_HOST)
    EXH_CUDA_TRY(cudaMemcpyAsync(type_out, dtype, sizeof(int) * (size_t)ng, cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    exh_set_error_msg("a galaxy flag names a halo outside the catalogue", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  return EXH_OK;
}
