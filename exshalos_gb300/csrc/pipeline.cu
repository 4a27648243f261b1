// Halo-box pipeline entry points: Generate_Halos_Box_from_Pk
// (src/exshalos/box.c:4-68, binding exshalos.c:710-940), Find_Halos on a
// given grid (exshalos.c:509-610), the Gaussian field alone
// (exshalos.c:46-121) and the result fetch.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.cuh"
#include "halos.cuh"
#include "lpt.cuh"
#include "pipeline.cuh"
#include "fft4.cuh"

using namespace exh;

namespace exh {
void halo_state_release(Ctx& c) { c.halos = HaloState(); }
}  // namespace exh

#define REQUIRE(cond, code, msg)                  \
  do {                                            \
    if (!(cond)) {                                \
      exh_set_error_msg(msg, __FILE__, __LINE__); \
      return code;                                \
    }                                             \
  } while (0)

static int check_common(const exh_halo_params* p, const float* k, const float* P, int Nk) {
  REQUIRE(p && k && P, EXH_E_INVALID, "null argument");
  REQUIRE(Nk >= 3, EXH_E_INVALID, "the P(k) table needs at least 3 points");
  REQUIRE(p->ndx >= 4 && p->ndy >= 4 && p->ndz >= 4 && p->ndx <= 1024 && p->ndy <= 1024 && p->ndz <= 1024,
          EXH_E_INVALID, "cells per side must be in [4, 1024]");
  REQUIRE((p->ndz % 2) == 0, EXH_E_INVALID, "ndz must be even");
  REQUIRE(p->Lc > 0.f && p->Lc < 100.f, EXH_E_INVALID, "cell size Lc must be in (0, 100) Mpc/h");
  REQUIRE(p->R_max >= 100000.f, EXH_E_UNSUPPORTED, "R_max < 1e5 (FFTLog truncation) is not built");
  REQUIRE(p->field_stream == EXH_FIELD_PHILOX || p->field_stream == EXH_FIELD_TAUS, EXH_E_INVALID,
          "unknown field stream");
  REQUIRE(p->OUT_PROF == 0, EXH_E_UNSUPPORTED, "Lagrangian profiles (OUT_PROF) are not built");
  for (int i = 0; i < Nk; i++) REQUIRE(k[i] > 0.f && P[i] >= 0.f, EXH_E_INVALID, "k must be > 0 and P >= 0");
  return EXH_OK;
}

namespace {

// Find_Halos (find_halos.c:479-563) on the device field `delta`
// order-independent 64-bit digest of a grid (sum of splitmix64 of value bits
// and index): a repeated grid is recognised without a host copy
__global__ void k_grid_hash(const float* __restrict__ d, size_t n, unsigned long long* __restrict__ out) {
  unsigned long long s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long x = ((unsigned long long)__float_as_uint(d[i]) << 32) ^ (unsigned long long)i;
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    s += x ^ (x >> 31);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

int grid_digest(Ctx& c, const float* d, size_t n, cudaStream_t st, unsigned long long* out) {
  EXH_TRY(c.buf[B_HOSTIO2].ensure(64));
  unsigned long long* dh = reinterpret_cast<unsigned long long*>(c.buf[B_HOSTIO2].as<char>() + 32);
  EXH_CUDA_TRY(cudaMemsetAsync(dh, 0, sizeof(unsigned long long), st));
  k_grid_hash<<<EXH_NUM_SMS * 8, 256, 0, st>>>(d, n, dh);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  EXH_CUDA_TRY(cudaMemcpyAsync(out, dh, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  *out |= 1ull;       // 0 stays "no digest"
  return EXH_OK;
}

// grid_hash != 0: the peaks and their sorted order of a grid with that
// digest are reused from the previous call (they do not depend on the
// barrier, the cosmology or Nmin), so repeated halo finding on one grid --
// barrier fits -- skips peak finding and the sort
int run_halo_finder(Ctx& c, const BoxParams& b, const float* k, const float* P, int Nk, int setup_fp64,
                    const float* delta, HaloDev* h, ShellTable* t, cudaStream_t st, unsigned long long grid_hash = 0) {
  HostTables& tab = c.halos.tab;
  // verbose >= 2: wall-clock milliseconds of each stage, the stream
  // synchronised at every mark (the stages wait on their counters anyway)
  auto t_mark = std::chrono::steady_clock::now();
  auto mark = [&](const char* what) -> int {
    if (c.verbose < 2) return EXH_OK;
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    const auto now = std::chrono::steady_clock::now();
    printf("  [%s: %.3f ms]\n", what, std::chrono::duration<double, std::milli>(now - t_mark).count());
    fflush(stdout);
    t_mark = now;
    return EXH_OK;
  };
  EXH_TRY(mark("before the halo finder"));
  // the tables depend on P(k), the cosmology, the cell and the barrier only:
  // reuse them across realisations (the key holds every input bit)
  std::string key;
  {
    const float scal[] = {b.Om0, b.redshift, b.dc, b.Lc, b.a, b.beta, b.alpha};
    key.append(reinterpret_cast<const char*>(scal), sizeof(scal));
    key.append(reinterpret_cast<const char*>(&setup_fp64), sizeof(int));
    key.append(reinterpret_cast<const char*>(k), sizeof(float) * Nk);
    key.append(reinterpret_cast<const char*>(P), sizeof(float) * Nk);
  }
  if (key != c.tab_key || c.tab_cache.Ncells == 0) {
    HostTables fresh;
    EXH_TRY(halo_tables(b, k, P, Nk, setup_fp64, fresh.Sig_grid, fresh.Btab, fresh.M, fresh.Int));
    fresh.Ncells = (int)fresh.Sig_grid.size();
    fresh.Nr = Nk;
    c.tab_cache = fresh;
    c.tab_key = key;
  }
  tab = c.tab_cache;
  EXH_TRY(build_shell_tables(c, b, tab.Ncells, t, st));
  EXH_TRY(c.buf[B_HOSTIO].ensure(sizeof(float) * tab.Ncells));
  float* Btab_dev = c.buf[B_HOSTIO].as<float>();
  EXH_CUDA_TRY(cudaMemcpyAsync(Btab_dev, tab.Btab.data(), sizeof(float) * tab.Ncells, cudaMemcpyHostToDevice, st));
  const bool reuse = grid_hash != 0 && grid_hash == c.peak_hash && c.peak_nd[0] == b.nd[0] &&
                     c.peak_nd[1] == b.nd[1] && c.peak_nd[2] == b.nd[2];
  if (reuse) {
    h->np = c.peak_np;
    h->key = c.peak_key;
    h->id = c.peak_id;
  } else {
    c.peak_hash = 0;
    EXH_TRY(mark("tables"));
    EXH_TRY(find_peaks(c, delta, b, h, st));
    if (c.verbose) { printf("There are %lld peaks\n", (long long)h->np); fflush(stdout); }
    EXH_TRY(mark("peaks"));
    EXH_TRY(sort_peaks(c, h, st));
    if (c.verbose) { printf("peaks sorted\n"); fflush(stdout); }
    EXH_TRY(mark("sort"));
    if (grid_hash != 0) {
      c.peak_hash = grid_hash;
      c.peak_nd[0] = b.nd[0]; c.peak_nd[1] = b.nd[1]; c.peak_nd[2] = b.nd[2];
      c.peak_np = h->np;
      c.peak_key = h->key;
      c.peak_id = h->id;
    }
  }
  HaloScalars hs;
  hs.Bmin = tab.Btab[tab.Ncells - 1];
  hs.Mtot = b.Mtot;
  hs.Ncells = tab.Ncells;
  hs.Nmin = b.Nmin;
  hs.nmin_half = b.nmin / 2;
  hs.n0 = b.nd[0]; hs.n1 = b.nd[1]; hs.n2 = b.nd[2];
  EXH_TRY(grow_halos(c, delta, b, hs, Btab_dev, *t, h, st));
  if (c.verbose) { printf("There are %lld halos\n", (long long)h->nh); fflush(stdout); }
  EXH_TRY(mark("growth"));
  const size_t nh = std::max<int64_t>(h->nh, 1);
  EXH_TRY(c.buf[B_MH].ensure((sizeof(float) + 4 * sizeof(int)) * nh));
  float* Mh = c.buf[B_MH].as<float>();
  int* cnt = reinterpret_cast<int*>(Mh + nh);
  int* xc = cnt + nh;
  EXH_TRY(halo_masses(c, b, *h, tab, Mh, cnt, xc, st));
  EXH_TRY(mark("masses"));
  HaloState& s = c.halos;
  s.nh = h->nh; s.np = h->np; s.nproc = h->nproc;
  s.nd[0] = b.nd[0]; s.nd[1] = b.nd[1]; s.nd[2] = b.nd[2];
  s.ng = b.ng;
  s.Mh = Mh; s.count = cnt; s.xc = xc;
  s.flag = h->flag; s.hid = h->hid;
  return EXH_OK;
}

__global__ void k_lagrangian_posh(const int* __restrict__ xc, int64_t nh, float Lc, float* __restrict__ posh) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 3 * nh) return;
  posh[i] = (float)((double)Lc * ((double)xc[i] + 0.5));     // exshalos.c:591
}

}  // namespace

extern "C" {

void exh_halo_params_default(exh_halo_params* p) {
  // defaults of Generate_Halos_Box_from_Pk, pyexshalos/mock.py:11-39
  std::memset(p, 0, sizeof(*p));
  p->R_max = 100000.f;
  p->ndx = p->ndy = p->ndz = 256;
  p->Lc = 2.f;
  p->seed = 12345;
  p->k_smooth = 10000.f;
  p->Om0 = 0.31f;
  p->redshift = 0.f;
  p->dc = -1.f;
  p->Nmin = 1;
  p->a = 1.f;
  p->beta = 0.f;
  p->alpha = 0.f;
  p->nthreads = 1;
  p->field_stream = EXH_FIELD_TAUS;      // the reference's realisation for a seed
  p->setup_fp64 = 0;
}

int exh_density_grid_compute(exh_ctx* ctx, const float* k, const float* P, int Nk, const exh_halo_params* prm,
                             float* delta, int mem, void* stream) {
  REQUIRE(ctx && delta, EXH_E_INVALID, "null argument");
  EXH_TRY(check_common(prm, k, P, Nk));
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  BoxParams b;
  // density_grid_compute sets a fixed cosmology (exshalos.c:71-73); only the box matters
  EXH_TRY(setup_box(&b, prm->ndx, prm->ndy, prm->ndz, prm->Lc, 0.31f, 0.f, 1.686f, 1, 1.f, 0.f, 0.f, prm->seed));
  float* d = delta;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_DELTA].ensure(sizeof(float) * b.ng));
    d = c.buf[B_DELTA].as<float>();
  }
  EXH_TRY(field_real(c, b, k, P, Nk, prm->field_stream, prm->fixed, prm->phase, d, st));
  if (mem == EXH_MEM_HOST) {
    EXH_CUDA_TRY(cudaMemcpyAsync(delta, d, sizeof(float) * b.ng, cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    EXH_TRY(taus_verify(c));
  }
  return EXH_OK;
}

int exh_halos_box_from_pk(exh_ctx* ctx, const float* k, const float* P, int Nk, const exh_halo_params* prm,
                          int64_t* nh_out, void* stream) {
  REQUIRE(ctx && nh_out, EXH_E_INVALID, "null argument");
  EXH_TRY(check_common(prm, k, P, Nk));
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  halo_state_release(c);
  c.verbose = prm->verbose;
  BoxParams b;
  EXH_TRY(setup_box(&b, prm->ndx, prm->ndy, prm->ndz, prm->Lc, prm->Om0, prm->redshift, prm->dc, prm->Nmin, prm->a,
                    prm->beta, prm->alpha, prm->seed));
  const size_t ng = b.ng;
  // field (box.c:18, k_smooth fixed at 1e5 there)
  float* A_dev = nullptr;
  EXH_TRY(upload_amplitudes(c, b, k, P, Nk, &A_dev, st));
  EXH_TRY(c.buf[B_DELTA].ensure(sizeof(float) * ng));
  float* delta = c.buf[B_DELTA].as<float>();
  FieldModes modes;
  EXH_TRY(make_field_modes(c, b, A_dev, prm->field_stream, prm->fixed, prm->phase, st, &modes));
  {
    FFTPlan3D* p;
    EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
    EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * (size_t)b.nd[0] * b.nd[1] * p->nc));
    FieldGen gen{modes};
    EXH_CUDA_TRY(fft_c2r_3d(*p, gen, c.buf[B_WORK].as<float2>(), RealPairStore{delta, b.nd[2], b.Normx}, st));
  }
  // LPT (box.c:38-58) depends on the field's modes only: it is enqueued on the
  // context's side stream, after the field, and runs beside the halo finder
  // (whose sort and growth are latency-bound and leave most SMs idle); the
  // halo sums wait for it.  The two share no buffer.
  cudaStream_t side;
  EXH_TRY(c.fork_stream(st, &side));
  EXH_TRY(c.buf[B_S].ensure(sizeof(float) * 3 * ng));
  EXH_TRY(c.buf[B_PHI1].ensure(sizeof(float) * ng));
  float* S = c.buf[B_S].as<float>();
  float* phi1 = c.buf[B_PHI1].as<float>();
  float* phi2 = nullptr;
  if (prm->DO_2LPT) {
    EXH_TRY(c.buf[B_PHI2].ensure(sizeof(float) * ng));
    phi2 = c.buf[B_PHI2].as<float>();
  }
  float* V = nullptr;
  if (prm->OUT_VEL) {
    EXH_TRY(c.buf[B_VEL].ensure(sizeof(float) * 3 * ng));
    V = c.buf[B_VEL].as<float>();
  }
  EXH_CUDA_TRY(cudaEventRecord(c.ev_fork, st));
  EXH_CUDA_TRY(cudaStreamWaitEvent(side, c.ev_fork, 0));
  EXH_TRY(lpt_run(c, b, modes, prm->k_smooth, prm->DO_2LPT != 0, S, V, phi1, phi2, side));
  EXH_CUDA_TRY(cudaEventRecord(c.ev_join, side));
  // halos (box.c:21)
  HaloDev h;
  ShellTable t;
  const int hs = run_halo_finder(c, b, k, P, Nk, prm->setup_fp64, delta, &h, &t, st);
  EXH_CUDA_TRY(cudaStreamWaitEvent(st, c.ev_join, 0));
  // the halo finder has synchronised the stream: the taus stream's count is in
  const int tv = taus_verify(c);
  if (hs != EXH_OK || tv != EXH_OK) {
    EXH_CUDA_TRY(cudaStreamSynchronize(side));      // nothing of this call left running on return
    return tv != EXH_OK ? tv : hs;
  }
  const size_t nh = std::max<int64_t>(h.nh, 1);
  EXH_TRY(c.buf[B_POSH].ensure(sizeof(float) * 6 * nh));
  float* posh = c.buf[B_POSH].as<float>();
  float* velh = prm->OUT_VEL ? posh + 3 * nh : nullptr;
  const HaloOut o = make_halo_out(b, posh, velh);
  EXH_TRY(halo_displacements(c, b, h, t, S, V, o, st));
  HaloState& s = c.halos;
  s.posh = posh;
  s.velh = velh;
  s.delta = prm->OUT_DEN ? delta : nullptr;
  if (prm->OUT_LPT) {
    EXH_TRY(c.buf[B_V].ensure(sizeof(float) * 6 * ng));
    float* pos = c.buf[B_V].as<float>();
    float* vel = prm->OUT_VEL ? pos + 3 * ng : nullptr;
    EXH_TRY(particles(b, S, V, o, pos, vel, st));
    s.pos = pos;
    s.vel = vel;
  }
  *nh_out = s.nh;
  return EXH_OK;
}

int exh_find_halos(exh_ctx* ctx, const float* delta, int ndx, int ndy, int ndz, const float* k, const float* P,
                   int Nk, const exh_halo_params* prm, int mem, int64_t* nh_out, void* stream) {
  REQUIRE(ctx && delta && nh_out && prm, EXH_E_INVALID, "null argument");
  exh_halo_params q = *prm;
  q.ndx = ndx; q.ndy = ndy; q.ndz = ndz;
  q.ndz += (ndz & 1);   // evenness only matters for the FFTs, not used here
  EXH_TRY(check_common(&q, k, P, Nk));
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  halo_state_release(c);
  c.verbose = prm->verbose;
  BoxParams b;
  // find_halos binds the mass draws to seed 12345 (exshalos.c:552)
  EXH_TRY(setup_box(&b, ndx, ndy, ndz, prm->Lc, prm->Om0, prm->redshift, prm->dc, prm->Nmin, prm->a, prm->beta,
                    prm->alpha, 12345));
  const float* d = delta;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_DELTA].ensure(sizeof(float) * b.ng));
    EXH_CUDA_TRY(cudaMemcpyAsync(c.buf[B_DELTA].p, delta, sizeof(float) * b.ng, cudaMemcpyHostToDevice, st));
    d = c.buf[B_DELTA].as<float>();
  }
  HaloDev h;
  ShellTable t;
  unsigned long long digest = 0;
  EXH_TRY(grid_digest(c, d, b.ng, st, &digest));
  EXH_TRY(run_halo_finder(c, b, k, P, Nk, prm->setup_fp64, d, &h, &t, st, digest));
  const size_t nh = std::max<int64_t>(h.nh, 1);
  EXH_TRY(c.buf[B_POSH].ensure(sizeof(float) * 6 * nh));
  float* posh = c.buf[B_POSH].as<float>();
  if (h.nh > 0) {
    k_lagrangian_posh<<<exh_div_up(3 * h.nh, 256), 256, 0, st>>>(c.halos.xc, h.nh, b.Lc, posh);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  c.halos.posh = posh;
  *nh_out = h.nh;
  return EXH_OK;
}

int exh_halos_box_from_grid(exh_ctx* ctx, const float* delta, int ndx, int ndy, int ndz, const float* k,
                            const float* P, int Nk, const float* S_in, const float* V_in, const exh_halo_params* prm,
                            int mem, int64_t* nh_out, void* stream) {
  REQUIRE(ctx && delta && nh_out && prm, EXH_E_INVALID, "null argument");
  REQUIRE(!(prm->OUT_VEL && S_in && !V_in), EXH_E_INVALID, "OUT_VEL with given displacements needs V");
  exh_halo_params q = *prm;
  q.ndx = ndx; q.ndy = ndy; q.ndz = ndz;
  EXH_TRY(check_common(&q, k, P, Nk));
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  halo_state_release(c);
  c.verbose = prm->verbose;
  BoxParams b;
  // halos_box_from_grid binds the mass draws to seed 1234 (exshalos.c:987)
  EXH_TRY(setup_box(&b, ndx, ndy, ndz, prm->Lc, prm->Om0, prm->redshift, prm->dc, prm->Nmin, prm->a, prm->beta,
                    prm->alpha, 1234));
  const size_t ng = b.ng;
  const float* d = delta;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_DELTA].ensure(sizeof(float) * ng));
    EXH_CUDA_TRY(cudaMemcpyAsync(c.buf[B_DELTA].p, delta, sizeof(float) * ng, cudaMemcpyHostToDevice, st));
    d = c.buf[B_DELTA].as<float>();
  }
  EXH_TRY(c.buf[B_S].ensure(sizeof(float) * 3 * ng));
  float* S = c.buf[B_S].as<float>();
  float* V = nullptr;
  if (prm->OUT_VEL) {
    EXH_TRY(c.buf[B_VEL].ensure(sizeof(float) * 3 * ng));
    V = c.buf[B_VEL].as<float>();
  }
  cudaStream_t side = nullptr;
  if (!S_in) {
    // box.c:108-143: delta_k = Normk r2c(delta), then 1LPT (and 2LPT), on the
    // side stream beside the halo finder (both only read the grid)
    EXH_TRY(c.buf[B_PHI1].ensure(sizeof(float) * ng));
    float* phi1 = c.buf[B_PHI1].as<float>();
    float* phi2 = nullptr;
    if (prm->DO_2LPT) {
      EXH_TRY(c.buf[B_PHI2].ensure(sizeof(float) * ng));
      phi2 = c.buf[B_PHI2].as<float>();
    }
    EXH_TRY(c.fork_stream(st, &side));
    EXH_CUDA_TRY(cudaEventRecord(c.ev_fork, st));
    EXH_CUDA_TRY(cudaStreamWaitEvent(side, c.ev_fork, 0));
    EXH_TRY(lpt_run_grid(c, b, d, prm->k_smooth, prm->DO_2LPT != 0, S, V, phi1, phi2, side));
    EXH_CUDA_TRY(cudaEventRecord(c.ev_join, side));
  }
  HaloDev h;
  ShellTable t;
  const int hs = run_halo_finder(c, b, k, P, Nk, prm->setup_fp64, d, &h, &t, st);
  if (side) EXH_CUDA_TRY(cudaStreamWaitEvent(st, c.ev_join, 0));
  if (hs != EXH_OK) {
    if (side) EXH_CUDA_TRY(cudaStreamSynchronize(side));
    return hs;
  }
  if (S_in) {
    // box.c:89-105: the given displacements (and velocities), [ng][3]
    const float* Sd = S_in;
    const float* Vd = V_in;
    if (mem == EXH_MEM_HOST) {
      EXH_TRY(c.buf[B_V].ensure(sizeof(float) * 6 * ng));
      float* stage = c.buf[B_V].as<float>();
      EXH_CUDA_TRY(cudaMemcpyAsync(stage, S_in, sizeof(float) * 3 * ng, cudaMemcpyHostToDevice, st));
      Sd = stage;
      if (V && V_in) {
        EXH_CUDA_TRY(cudaMemcpyAsync(stage + 3 * ng, V_in, sizeof(float) * 3 * ng, cudaMemcpyHostToDevice, st));
        Vd = stage + 3 * ng;
      }
    }
    EXH_TRY(aos_to_planes(Sd, ng, S, st));
    if (V) EXH_TRY(aos_to_planes(Vd, ng, V, st));
  }
  const size_t nh = std::max<int64_t>(h.nh, 1);
  EXH_TRY(c.buf[B_POSH].ensure(sizeof(float) * 6 * nh));
  float* posh = c.buf[B_POSH].as<float>();
  float* velh = prm->OUT_VEL ? posh + 3 * nh : nullptr;
  const HaloOut o = make_halo_out(b, posh, velh);
  EXH_TRY(halo_displacements(c, b, h, t, S, V, o, st));
  HaloState& s = c.halos;
  s.posh = posh;
  s.velh = velh;
  if (prm->OUT_LPT) {
    // particle positions q + S wrapped (lpt.c:229-242); with given
    // displacements the reference leaves its output array unset
    // (exshalos.c:1001-1013), here it is filled the same way
    EXH_TRY(c.buf[B_V].ensure(sizeof(float) * 6 * ng));
    float* pos = c.buf[B_V].as<float>();
    float* vel = prm->OUT_VEL ? pos + 3 * ng : nullptr;
    EXH_TRY(particles(b, S, V, o, pos, vel, st));
    s.pos = pos;
    s.vel = vel;
  }
  *nh_out = s.nh;
  return EXH_OK;
}

int exh_halos_fetch(exh_ctx* ctx, float* posh, float* velh, float* Mh, int32_t* xc, int32_t* count, float* grid,
                    float* pos, float* vel, int64_t* flag, int mem, void* stream) {
  REQUIRE(ctx, EXH_E_INVALID, "null context");
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  const HaloState& s = c.halos;
  const cudaMemcpyKind kind = mem == EXH_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  const size_t nh = (size_t)s.nh, ng = s.ng;
  REQUIRE(!velh || s.velh || nh == 0, EXH_E_INVALID, "velocities were not requested (OUT_VEL)");
  REQUIRE(!grid || s.delta, EXH_E_INVALID, "the field was not requested (OUT_DEN)");
  REQUIRE(!pos || s.pos, EXH_E_INVALID, "particles were not requested (OUT_LPT)");
  REQUIRE(!vel || s.vel, EXH_E_INVALID, "particle velocities were not requested (OUT_LPT and OUT_VEL)");
  if (nh) {
    if (posh) EXH_CUDA_TRY(cudaMemcpyAsync(posh, s.posh, sizeof(float) * 3 * nh, kind, st));
    if (velh) EXH_CUDA_TRY(cudaMemcpyAsync(velh, s.velh, sizeof(float) * 3 * nh, kind, st));
    if (Mh) EXH_CUDA_TRY(cudaMemcpyAsync(Mh, s.Mh, sizeof(float) * nh, kind, st));
    if (xc) EXH_CUDA_TRY(cudaMemcpyAsync(xc, s.xc, sizeof(int) * 3 * nh, kind, st));
    if (count) EXH_CUDA_TRY(cudaMemcpyAsync(count, s.count, sizeof(int) * nh, kind, st));
  }
  if (grid) EXH_CUDA_TRY(cudaMemcpyAsync(grid, s.delta, sizeof(float) * ng, kind, st));
  if (pos) EXH_CUDA_TRY(cudaMemcpyAsync(pos, s.pos, sizeof(float) * 3 * ng, kind, st));
  if (vel) EXH_CUDA_TRY(cudaMemcpyAsync(vel, s.vel, sizeof(float) * 3 * ng, kind, st));
  if (flag) {
    REQUIRE(s.flag, EXH_E_INVALID, "no halo flags available");
    int64_t* fdev = flag;
    if (mem == EXH_MEM_HOST) {
      EXH_TRY(c.buf[B_HOSTIO].ensure(sizeof(int64_t) * ng));
      fdev = c.buf[B_HOSTIO].as<int64_t>();
    }
    HaloDev hd;
    hd.flag = s.flag;
    hd.hid = s.hid;
    EXH_TRY(flags_to_reference(hd, ng, fdev, st));
    if (mem == EXH_MEM_HOST) EXH_CUDA_TRY(cudaMemcpyAsync(flag, fdev, sizeof(int64_t) * ng, kind, st));
  }
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  return EXH_OK;
}

int exh_halo_tables(exh_ctx* ctx, int* Ncells, int* Nr, float* Sig_grid, float* Btab, double* M, double* Int) {
  REQUIRE(ctx && Ncells && Nr, EXH_E_INVALID, "null argument");
  const HostTables& t = ctx->c.halos.tab;
  *Ncells = t.Ncells;
  *Nr = t.Nr;
  if (Sig_grid && t.Ncells) std::memcpy(Sig_grid, t.Sig_grid.data(), sizeof(float) * t.Ncells);
  if (Btab && t.Ncells) std::memcpy(Btab, t.Btab.data(), sizeof(float) * t.Ncells);
  if (M && t.Nr) std::memcpy(M, t.M.data(), sizeof(double) * t.Nr);
  if (Int && t.Nr) std::memcpy(Int, t.Int.data(), sizeof(double) * t.Nr);
  return EXH_OK;
}

}  // extern "C"
