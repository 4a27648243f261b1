// Halo-box pipeline entry points: Generate_Halos_Box_from_Pk
// (src/exshalos/box.c:4-68) and its sub-stage hooks.
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "pipeline.cuh"

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
  REQUIRE(p->field_stream == EXH_FIELD_PHILOX, EXH_E_UNSUPPORTED, "unknown field stream");
  return EXH_OK;
}

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
  p->field_stream = EXH_FIELD_PHILOX;
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
  EXH_TRY(setup_box(&b, prm->ndx, prm->ndy, prm->ndz, prm->Lc, 0.31f, 0.f, 1.686f, 1, 1.f, 0.f, 0.f, prm->seed));
  float* d = delta;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_DELTA].ensure(sizeof(float) * b.ng));
    d = c.buf[B_DELTA].as<float>();
  }
  EXH_TRY(field_real(c, b, k, P, Nk, prm->fixed, prm->phase, d, st));
  if (mem == EXH_MEM_HOST) {
    EXH_CUDA_TRY(cudaMemcpyAsync(delta, d, sizeof(float) * b.ng, cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return EXH_OK;
}

int exh_halos_box_from_pk(exh_ctx* ctx, const float* k, const float* P, int Nk, const exh_halo_params* prm,
                          int64_t* nh_out, void* stream) {
  (void)ctx; (void)k; (void)P; (void)Nk; (void)prm; (void)nh_out; (void)stream;
  exh_set_error_msg("halo pipeline not built yet", __FILE__, __LINE__);
  return EXH_E_UNSUPPORTED;
}

int exh_find_halos(exh_ctx* ctx, const float* delta, int ndx, int ndy, int ndz, const float* k, const float* P,
                   int Nk, const exh_halo_params* prm, int mem, int64_t* nh_out, void* stream) {
  (void)ctx; (void)delta; (void)ndx; (void)ndy; (void)ndz; (void)k; (void)P; (void)Nk; (void)prm; (void)mem;
  (void)nh_out; (void)stream;
  exh_set_error_msg("halo finder not built yet", __FILE__, __LINE__);
  return EXH_E_UNSUPPORTED;
}

int exh_halos_fetch(exh_ctx* ctx, float* posh, float* velh, float* Mh, int32_t* xc, int32_t* count, float* grid,
                    float* pos, float* vel, int64_t* flag, int mem, void* stream) {
  (void)ctx; (void)posh; (void)velh; (void)Mh; (void)xc; (void)count; (void)grid; (void)pos; (void)vel; (void)flag;
  (void)mem; (void)stream;
  return EXH_E_UNSUPPORTED;
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
