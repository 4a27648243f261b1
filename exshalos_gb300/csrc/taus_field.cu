// The reference's Gaussian-field stream on the GPU (Compute_Den,
// src/exshalos/density_grid.c:88-186): one gsl_rng_taus stream seeded with
// the realisation's seed, consumed in the mode loop's order (i, j, k over the
// half-complex grid, Hermitian copies drawing nothing), two gsl_ran_gaussian
// deviates per mode (one for the eight self-conjugate modes), or with
// `fixed` one gsl_ran_flat phase per mode (none for the self-conjugate ones).
//
// gsl_ran_gaussian is the Marsaglia polar method: x = -1 + 2 u1, y = -1 + 2 u2
// from two gsl_rng_uniform_pos draws (which skip a raw value of 0), rejected
// while r2 = x^2 + y^2 > 1 or r2 == 0, then y sqrt(-2 ln r2 / r2).  Each
// deviate therefore takes an accepted pair of the zero-filtered stream, and
// the k-th deviate of the field is the k-th accepted pair.  Here:
//  1. chunks of TF_CHUNK raw values (one thread each, its state by GF(2)
//     jump-ahead) count their zeros and their accepted pairs for both
//     parities of the filtered index at the chunk start (a pair belongs to
//     the chunk that holds its first value; the last one may end in the
//     next chunk);
//  2. two prefix sums give each chunk its parity (zeros before it) and the
//     number of accepted pairs before it;
//  3. the chunks walk their values again and write each accepted pair's
//     deviate at its index.
// The acceptance test is exact in 64-bit integers (x = a / 2^31 with a an
// integer) except within 2^-50 of the unit circle, where the reference's
// double operations (no fused multiply-add) decide.  The reference rounds its
// FP64 deviate to float (density_grid.c:182-183); here that float comes from
// a double-float evaluation wherever that decides it, and from the FP64
// formula for the rest (taus_chunk.h).
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "ctx.cuh"
#include "field.cuh"
#include "lpt.cuh"
#include "scan.cuh"
#include "taus.cuh"
#include "taus_chunk.h"
#include "timing.cuh"

namespace exh {

namespace {

constexpr int TF_CHUNK = 64;      // raw values per thread (even): short chunks, many warps for the
                                  // dependent double-float chains of the deviates
constexpr int TF_T = 256;

// columns of J^(TF_CHUNK l) for the lane offsets l = 0..31 of a warp's
// chunks, per component (host: from the power-of-two jump matrices)
struct LaneJump {
  unsigned col[3][32][32];
};

const LaneJump& lane_jump_host() {
  static const LaneJump LJ = [] {
    const TausJump& J = taus_jump_host();
    LaneJump t;
    for (int c = 0; c < 3; c++)
      for (int l = 0; l < 32; l++)
        for (int q = 0; q < 32; q++) {
          unsigned v = 1u << q;                              // image of bit q under J^(TF_CHUNK l)
          const unsigned long long n = (unsigned long long)TF_CHUNK * l;
          for (int e = 0; e < 32; e++)
            if ((n >> e) & 1ull) {
              unsigned acc = 0;
              for (int r = 0; r < 32; r++)
                if ((v >> r) & 1u) acc ^= J.col[c][e][r];
              v = acc;
            }
          t.col[c][l][q] = v;
        }
    return t;
  }();
  return LJ;
}

// y = M s over GF(2) by the whole warp: lane q contributes column q
__device__ __forceinline__ unsigned gf2_warp(const unsigned* __restrict__ col, unsigned s, unsigned lane) {
  unsigned v = ((s >> lane) & 1u) ? __ldg(col + lane) : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v ^= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned gf2_apply_row(const unsigned* col, unsigned s) {
  unsigned acc = 0;
#pragma unroll 8
  for (int q = 0; q < 32; q++)
    if ((s >> q) & 1u) acc ^= col[q];
  return acc;
}

// lane offset matrices in shared memory, rows padded to 33 words (lane l
// reads word l * 33 + q: conflict-free)
struct LaneJumpSmem {
  unsigned col[3][32][33];
};

__device__ __forceinline__ void load_lane_jump(const LaneJump* __restrict__ LJ, LaneJumpSmem* sL) {
  for (int q = threadIdx.x; q < 3 * 32 * 32; q += blockDim.x) {
    const int c = q >> 10, l = (q >> 5) & 31, r = q & 31;
    sL->col[c][l][r] = LJ->col[c][l][r];
  }
}

// state at the start of chunk `first + lane` for every lane of a warp
// (all 32 lanes call this together): the warp jumps to chunk `first`
// cooperatively, then each lane applies its lane-offset matrix
__device__ __forceinline__ void chunk_state(const TausJump* __restrict__ J, const LaneJumpSmem* sL, TausState s0,
                                            unsigned long long first, unsigned s[3]) {
  const unsigned lane = threadIdx.x & 31;
  s[0] = s0.s[0]; s[1] = s0.s[1]; s[2] = s0.s[2];
  const unsigned long long n = first * TF_CHUNK;
  for (int e = 0; e < 32; e++)
    if ((n >> e) & 1ull)
      for (int c = 0; c < 3; c++) s[c] = gf2_warp(J->col[c][e], s[c], lane);
  for (int c = 0; c < 3; c++) s[c] = gf2_apply_row(sL->col[c][lane], s[c]);
}

struct TausNext {
  unsigned s[3];   // the stream's state
  __device__ __forceinline__ unsigned operator()() { return taus_next(s); }
};

__global__ void __launch_bounds__(TF_T) k_taus_count(const TausJump* __restrict__ J,
                                                     const LaneJump* __restrict__ LJ, TausState s0, int nch,
                                                     unsigned* __restrict__ zc, unsigned* __restrict__ a0,
                                                     unsigned* __restrict__ a1) {
  __shared__ LaneJumpSmem sL;
  load_lane_jump(LJ, &sL);
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  TausNext g;
  chunk_state(J, &sL, s0, (unsigned long long)(c & ~31), g.s);
  if (c >= nch) return;
  polar_chunk_count(g, TF_CHUNK, &zc[c], &a0[c], &a1[c]);
}

__global__ void k_taus_select(const unsigned* __restrict__ zbefore, const unsigned* __restrict__ a0,
                              const unsigned* __restrict__ a1, int nch, unsigned* __restrict__ sel) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nch) sel[c] = (zbefore[c] & 1u) ? a1[c] : a0[c];
}

// ln(c_i) and 1 / c_i of the double-float logarithm's table points
// c_i = 0.75 + (i + 1/2) / 256 (taus_chunk.h), as float pairs
constexpr int TF_TAB = 2 * 192;

struct LogTables {
  float lnc[TF_TAB], invc[TF_TAB];
};

const LogTables& log_tables_host() {
  static const LogTables T = [] {
    LogTables t;
    for (int i = 0; i < 192; i++) {
      const double c = 0.75 + (i + 0.5) / 256.0, l = std::log(c), r = 1.0 / c;
      t.lnc[2 * i] = (float)l;
      t.lnc[2 * i + 1] = (float)(l - (double)t.lnc[2 * i]);
      t.invc[2 * i] = (float)r;
      t.invc[2 * i + 1] = (float)(r - (double)t.invc[2 * i]);
    }
    return t;
  }();
  return T;
}

// each accepted pair's float deviate: in double-float arithmetic where that
// decides the float, else in FP64 as the reference forms it
struct DeviateOut {
  float* out;
  long long idx, G;
  const float* lnc;
  const float* invc;
  __device__ __forceinline__ bool operator()(unsigned v1, unsigned v2) {
    if (idx >= G) return false;
    int undecided;
    float f = polar_deviate_f32(v1, v2, lnc, invc, &undecided);
    if (undecided) f = __double2float_rn(polar_deviate(v1, v2, [](double r) { return log(r); }));
    out[idx++] = f;
    return true;
  }
};

__global__ void __launch_bounds__(TF_T) k_taus_deviates(const TausJump* __restrict__ J,
                                                        const LaneJump* __restrict__ LJ,
                                                        const LogTables* __restrict__ tab, TausState s0, int nch,
                                                        const unsigned* __restrict__ zbefore,
                                                        const unsigned* __restrict__ abefore, long long G,
                                                        float* __restrict__ out) {
  __shared__ LaneJumpSmem sL;
  __shared__ LogTables sT;
  for (int q = threadIdx.x; q < TF_TAB; q += blockDim.x) {
    sT.lnc[q] = tab->lnc[q];
    sT.invc[q] = tab->invc[q];
  }
  load_lane_jump(LJ, &sL);
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  TausNext g;
  chunk_state(J, &sL, s0, (unsigned long long)(c & ~31), g.s);
  if (c >= nch) return;
  DeviateOut emit{out, (long long)abefore[c], G, sT.lnc, sT.invc};
  if (emit.idx >= G) return;
  polar_chunk_pairs(g, TF_CHUNK, zbefore[c] & 1u, emit);
}

// fixed amplitudes: one gsl_ran_flat(0, 2 pi) phase per draw, a (1 - u) + b u
// with a = 0, rounded to float as the reference stores theta
__global__ void __launch_bounds__(TF_T) k_taus_phases(const TausJump* __restrict__ J,
                                                      const LaneJump* __restrict__ LJ, TausState s0, long long G,
                                                      float* __restrict__ out) {
  __shared__ LaneJumpSmem sL;
  load_lane_jump(LJ, &sL);
  __syncthreads();
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  unsigned s[3];
  chunk_state(J, &sL, s0, (unsigned long long)(c & ~31ll), s);
  const long long d0 = c * TF_CHUNK;
  if (d0 >= G) return;
  const double two_pi = 2.0 * 3.14159265358979323846;
  for (int t = 0; t < TF_CHUNK && d0 + t < G; t++) {
    const double u = (double)taus_next(s) * (1.0 / 4294967296.0);
    out[d0 + t] = __double2float_rn(__dmul_rn(two_pi, u));
  }
}

// The draws of one (box, seed, fixed) are the same in every context, and a
// mock realisation draws them in two (the halo finder's and the smoothing
// ladder's, which run side by side).  Each context therefore offers the draws
// of its last seed to the other contexts of the process on the same device:
// an entry holds its device pointers (B_GAUSS and the accepted-pair count in
// B_TAUS), an event recorded on the producing stream once they are written,
// and one event per copy taken from them.  A context that needs the draws of
// an offered key waits on that event and copies them (one device-to-device
// copy instead of the three passes); a context rewrites or frees its own
// buffers only after withdrawing its entry and ordering its stream after
// every copy taken (a host wait where the buffers are reallocated).
struct TausOffer {
  const Ctx* owner = nullptr;
  int device = 0;
  std::string key;
  const float* draws = nullptr;
  size_t bytes = 0;
  const unsigned* have_dev = nullptr;   // accepted pairs (nullptr for phases)
  long long need = 0;
  cudaEvent_t ready = nullptr;
  std::vector<cudaEvent_t> reads;
};

std::mutex g_offer_mu;
std::vector<TausOffer> g_offers;

// withdraw c's offer; `st` (or, with host_wait, the host) waits for every
// copy taken from it
int offer_withdraw(const Ctx& c, cudaStream_t st, bool host_wait) {
  std::lock_guard<std::mutex> lk(g_offer_mu);
  for (size_t i = 0; i < g_offers.size(); i++) {
    TausOffer& o = g_offers[i];
    if (o.owner != &c) continue;
    cudaError_t e = cudaSuccess;
    for (cudaEvent_t ev : o.reads) {
      const cudaError_t ei = host_wait ? cudaEventSynchronize(ev) : cudaStreamWaitEvent(st, ev, 0);
      if (e == cudaSuccess) e = ei;
      cudaEventDestroy(ev);
    }
    cudaEventDestroy(o.ready);
    g_offers.erase(g_offers.begin() + (long)i);
    EXH_CUDA_TRY(e);
    return EXH_OK;
  }
  return EXH_OK;
}

// offer c's draws of `key`, written on `st`
int offer_publish(const Ctx& c, const std::string& key, const float* draws, size_t bytes, const unsigned* have_dev,
                  long long need, cudaStream_t st) {
  cudaEvent_t ev = nullptr;
  EXH_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  const cudaError_t e = cudaEventRecord(ev, st);
  if (e != cudaSuccess) {
    cudaEventDestroy(ev);
    EXH_CUDA_TRY(e);
  }
  TausOffer o;
  o.owner = &c;
  o.device = c.device;
  o.key = key;
  o.draws = draws;
  o.bytes = bytes;
  o.have_dev = have_dev;
  o.need = need;
  o.ready = ev;
  std::lock_guard<std::mutex> lk(g_offer_mu);
  g_offers.push_back(std::move(o));
  return EXH_OK;
}

// copy another context's offered draws of `key` into dev on `st`; *taken is
// false when no context of this device offers them
int offer_take(Ctx& c, const std::string& key, float* dev, size_t bytes, cudaStream_t st, bool* taken) {
  *taken = false;
  std::lock_guard<std::mutex> lk(g_offer_mu);
  for (TausOffer& o : g_offers) {
    if (o.owner == &c || o.device != c.device || o.key != key || o.bytes != bytes) continue;
    // copies that have completed need no further wait
    size_t w = 0;
    for (size_t r = 0; r < o.reads.size(); r++) {
      if (cudaEventQuery(o.reads[r]) == cudaSuccess) {
        cudaEventDestroy(o.reads[r]);
      } else {
        o.reads[w++] = o.reads[r];
      }
    }
    o.reads.resize(w);
    cudaGetLastError();
    if (o.have_dev && !c.taus_have_host)
      EXH_CUDA_TRY(cudaHostAlloc((void**)&c.taus_have_host, sizeof(unsigned), 0));
    cudaEvent_t rd = nullptr;
    EXH_CUDA_TRY(cudaEventCreateWithFlags(&rd, cudaEventDisableTiming));
    cudaError_t e = cudaStreamWaitEvent(st, o.ready, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dev, o.draws, bytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && o.have_dev)
      e = cudaMemcpyAsync(c.taus_have_host, o.have_dev, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaEventRecord(rd, st);
    if (e != cudaSuccess) {
      // the copy may have been enqueued: the owner must still wait for it
      cudaEventDestroy(rd);
      cudaStreamSynchronize(st);
      EXH_CUDA_TRY(e);
    }
    o.reads.push_back(rd);
    if (o.have_dev) {
      c.taus_need = o.need;
      c.taus_pending = true;
    }
    *taken = true;
    return EXH_OK;
  }
  return EXH_OK;
}

}  // namespace

void taus_offer_release(Ctx& c) { offer_withdraw(c, nullptr, true); }

int taus_field_draws(Ctx& c, const BoxParams& b, int fixed, cudaStream_t st, const float** out) {
  const int n0 = b.nd[0], n1 = b.nd[1], n2 = b.nd[2];
  const long long G = taus_draw_total(n0, n1, n2, fixed);
  std::string key;
  const int kv[5] = {n0, n1, n2, b.seed, fixed};
  key.append(reinterpret_cast<const char*>(kv), sizeof(kv));
  const size_t gbytes = sizeof(float) * (size_t)G;
  if (key == c.taus_key && c.buf[B_GAUSS].cap >= gbytes) {
    *out = c.buf[B_GAUSS].as<float>();         // the draws of this seed and box are there already
    return EXH_OK;
  }
  c.taus_key.clear();
  const size_t jbytes = (sizeof(TausJump) + sizeof(LaneJump) + sizeof(LogTables) + 255) / 256 * 256;
  const double p = M_PI / 4.0;                 // polar-method acceptance
  const long long pairs = fixed ? 0 : (long long)std::ceil(G / p + 12.0 * std::sqrt(G * (1.0 - p)) / p + 64.0);
  const long long nraw = fixed ? G : 2 * pairs;
  const int nch = (int)((nraw + TF_CHUNK - 1) / TF_CHUNK);
  const size_t nsc = (size_t)nch / SCAN_TILE + 2;
  const size_t tbytes = jbytes + sizeof(unsigned) * (6 * (size_t)nch + 2 * nsc + 4);
  // another context may still be copying this context's previous draws:
  // order this stream after those copies (the host, where a buffer is
  // about to be freed and reallocated)
  EXH_TRY(offer_withdraw(c, st, gbytes > c.buf[B_GAUSS].cap || tbytes > c.buf[B_TAUS].cap));
  EXH_TRY(c.buf[B_GAUSS].ensure(gbytes));
  float* dev = c.buf[B_GAUSS].as<float>();
  *out = dev;
  bool taken = false;
  EXH_TRY(offer_take(c, key, dev, gbytes, st, &taken));
  if (taken) {
    c.taus_key = key;
    return EXH_OK;
  }
  EXH_TRY(c.buf[B_TAUS].ensure(tbytes));
  TausJump* dJ = c.buf[B_TAUS].as<TausJump>();
  LaneJump* dL = reinterpret_cast<LaneJump*>(dJ + 1);
  LogTables* dT = reinterpret_cast<LogTables*>(dL + 1);
  if (c.taus_jump_at != (const void*)dJ) {     // first use, or the buffer was reallocated
    // the host tables have static storage: the copies may complete later
    EXH_CUDA_TRY(cudaMemcpyAsync(dJ, &taus_jump_host(), sizeof(TausJump), cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaMemcpyAsync(dL, &lane_jump_host(), sizeof(LaneJump), cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaMemcpyAsync(dT, &log_tables_host(), sizeof(LogTables), cudaMemcpyHostToDevice, st));
    c.taus_jump_at = dJ;
  }
  TausState s0;
  taus_seed_state((unsigned long)(unsigned)b.seed, s0.s);
  KTimer kt(KC_OTHER, st, sizeof(float) * (double)G);
  if (fixed) {
    const unsigned nb = exh_div_up((size_t)((G + TF_CHUNK - 1) / TF_CHUNK), TF_T);
    k_taus_phases<<<nb, TF_T, 0, st>>>(dJ, dL, s0, G, dev);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
    EXH_TRY(offer_publish(c, key, dev, gbytes, nullptr, 0, st));
    c.taus_key = key;
    return EXH_OK;
  }
  unsigned* zc = reinterpret_cast<unsigned*>(c.buf[B_TAUS].as<char>() + jbytes);
  unsigned* a0 = zc + nch;
  unsigned* a1 = a0 + nch;
  unsigned* zb = a1 + nch;
  unsigned* sel = zb + nch;
  unsigned* ab = sel + nch;
  unsigned* scr = ab + nch;
  unsigned* tot = scr + 2 * nsc;
  const unsigned nb = exh_div_up((size_t)nch, TF_T);
  k_taus_count<<<nb, TF_T, 0, st>>>(dJ, dL, s0, nch, zc, a0, a1);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  EXH_CUDA_TRY(exclusive_scan<unsigned>(zc, zb, (size_t)nch, scr, tot, st));
  k_taus_select<<<exh_div_up((size_t)nch, 256), 256, 0, st>>>(zb, a0, a1, nch, sel);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  EXH_CUDA_TRY(exclusive_scan<unsigned>(sel, ab, (size_t)nch, scr, tot + 1, st));
  k_taus_deviates<<<nb, TF_T, 0, st>>>(dJ, dL, dT, s0, nch, zb, ab, G, dev);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  // the stream was sized 12 standard deviations beyond the expected number
  // of pairs (a shortfall has probability below 1e-30); the count of
  // accepted pairs goes to pinned host memory and taus_verify() checks it at
  // the caller's next synchronisation, so this call does not wait
  if (!c.taus_have_host) EXH_CUDA_TRY(cudaHostAlloc((void**)&c.taus_have_host, sizeof(unsigned), 0));
  EXH_CUDA_TRY(cudaMemcpyAsync(c.taus_have_host, tot + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  c.taus_need = G;
  c.taus_pending = true;
  EXH_TRY(offer_publish(c, key, dev, gbytes, tot + 1, G, st));
  c.taus_key = key;
  return EXH_OK;
}

int taus_verify(Ctx& c) {
  if (!c.taus_pending) return EXH_OK;
  c.taus_pending = false;
  if ((long long)*c.taus_have_host < c.taus_need) {
    c.taus_key.clear();
    exh_set_error_msg("taus field stream: too few accepted pairs in the generated stream", __FILE__, __LINE__);
    return EXH_E_RANGE;
  }
  return EXH_OK;
}

}  // namespace exh
