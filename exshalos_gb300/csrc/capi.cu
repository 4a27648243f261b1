// C ABI entry points (include/exh_gb300.h): argument checks, host/device
// staging and dispatch to the stage drivers.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "ctx.cuh"
#include "lpt.cuh"
#include "spectrum.cuh"
#include "pipeline.cuh"

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void exh_set_error_msg(const char* msg, const char* file, int line) {
  char buf[512];
  const char* base = strrchr(file, '/');
  snprintf(buf, sizeof(buf), "%s (%s:%d)", msg, base ? base + 1 : file, line);
  g_last_error = buf;
}

namespace exh {
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace exh

using namespace exh;

#define REQUIRE(cond, code, msg)                          \
  do {                                                    \
    if (!(cond)) {                                        \
      exh_set_error_msg(msg, __FILE__, __LINE__);         \
      return code;                                        \
    }                                                     \
  } while (0)

extern "C" {

const char* exh_last_error(void) { return g_last_error.c_str(); }

const char* exh_strerror(int code) {
  switch (code) {
    case EXH_OK: return "ok";
    case EXH_E_INVALID: return "invalid argument";
    case EXH_E_NOMEM: return "out of memory";
    case EXH_E_CUDA: return "CUDA error";
    case EXH_E_RANGE: return "value outside the halo-finder tables";
    case EXH_E_TIMEOUT: return "device wait timed out";
    case EXH_E_UNSUPPORTED: return "option not supported";
    case EXH_E_NO_DEVICE: return "no CUDA device";
    default: return "unknown error";
  }
}

int exh_version(void) { return 100; }
int exh_check_precision(void) { return (int)sizeof(float); }
int64_t exh_launch_count(exh_ctx*) { return (int64_t)g_launches.load(); }

int exh_ctx_create(int device, exh_ctx** out) {
  REQUIRE(out, EXH_E_INVALID, "null output pointer");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    exh_set_error_msg("no CUDA device available", __FILE__, __LINE__);
    return EXH_E_NO_DEVICE;
  }
  REQUIRE(device >= 0 && device < n, EXH_E_INVALID, "device index out of range");
  EXH_CUDA_TRY(cudaSetDevice(device));
  exh_ctx* c = new (std::nothrow) exh_ctx();
  REQUIRE(c, EXH_E_NOMEM, "host allocation failed");
  c->c.device = device;
  *out = c;
  return EXH_OK;
}

int exh_ctx_destroy(exh_ctx* ctx) {
  if (!ctx) return EXH_OK;
  cudaSetDevice(ctx->c.device);
  taus_offer_release(ctx->c);        // no other context starts a copy from its buffers after this
  cudaDeviceSynchronize();
  for (size_t i = 0; i < ctx->c.lane_ctx.size(); i++) {
    exh_ctx_destroy(ctx->c.lane_ctx[i]);
    cudaStreamDestroy(ctx->c.lane_st[i]);
  }
  for (auto& kv : ctx->c.plans) fft_plan_destroy(&kv.second);
  if (ctx->c.ladder_graph) cudaGraphExecDestroy(ctx->c.ladder_graph);
  if (ctx->c.sort_graph) cudaGraphExecDestroy(ctx->c.sort_graph);
  if (ctx->c.sort_graph_src) cudaGraphDestroy(ctx->c.sort_graph_src);
  for (auto& e : ctx->c.grow_graphs) {
    cudaGraphExecDestroy(e.exec);
    cudaGraphDestroy(e.src);
  }
  if (ctx->c.capture) cudaStreamDestroy(ctx->c.capture);
  if (ctx->c.side) {
    cudaEventDestroy(ctx->c.ev_fork);
    cudaEventDestroy(ctx->c.ev_join);
    cudaStreamDestroy(ctx->c.side);
  }
  for (int i = 0; i < B_COUNT; i++) ctx->c.buf[i].release();
  if (ctx->c.taus_have_host) cudaFreeHost(ctx->c.taus_have_host);
  diff_state_release(ctx->c);
  halo_state_release(ctx->c);
  delete ctx;
  return EXH_OK;
}

int exh_grid_compute(exh_ctx* ctx, const float* pos, int64_t np, int nd, float L, int window, int folds,
                     float* grid, int mem, void* stream) {
  REQUIRE(ctx && grid, EXH_E_INVALID, "null context or grid");
  REQUIRE(np >= 0 && (np == 0 || pos), EXH_E_INVALID, "bad tracer array");
  REQUIRE(nd >= 2 && nd <= 1024, EXH_E_INVALID, "nd must be in [2, 1024]");
  REQUIRE(L > 0.f && folds >= 1, EXH_E_INVALID, "L must be positive and folds >= 1");
  REQUIRE(window == 2, EXH_E_UNSUPPORTED, "only the CIC window (2) is built");
  REQUIRE(folds == 1, EXH_E_UNSUPPORTED, "folded boxes are not built");
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t ng = (size_t)nd * nd * nd;
  const float* pos_d = pos;
  float* grid_d = grid;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_HOSTIO].ensure(sizeof(float) * 3 * (size_t)(np > 0 ? np : 1)));
    EXH_TRY(c.buf[B_GRID].ensure(sizeof(float) * ng));
    if (np > 0)
      EXH_CUDA_TRY(cudaMemcpyAsync(c.buf[B_HOSTIO].p, pos, sizeof(float) * 3 * np, cudaMemcpyHostToDevice, st));
    pos_d = c.buf[B_HOSTIO].as<float>();
    grid_d = c.buf[B_GRID].as<float>();
  }
  EXH_TRY(cic_assign(c, pos_d, np, nd, L, grid_d, st));
  if (mem == EXH_MEM_HOST) {
    EXH_CUDA_TRY(cudaMemcpyAsync(grid, grid_d, sizeof(float) * ng, cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return EXH_OK;
}

int exh_power_compute(exh_ctx* ctx, const float* grid, int nd, float L, int window, int Nk, float k_min,
                      float k_max, float* k_out, float* P_out, int64_t* count_out, int mem, void* stream) {
  REQUIRE(ctx && grid && k_out && P_out && count_out, EXH_E_INVALID, "null argument");
  REQUIRE(nd >= 4 && nd <= 1024 && (nd % 2) == 0, EXH_E_INVALID, "nd must be even in [4, 1024]");
  REQUIRE(Nk >= 1 && Nk <= 4096, EXH_E_INVALID, "Nk must be in [1, 4096]");
  REQUIRE(L > 0.f && k_max > k_min, EXH_E_INVALID, "need L > 0 and k_max > k_min");
  REQUIRE(window >= 0 && window <= 2, EXH_E_UNSUPPORTED, "windows 0 (none), 1 (NGP), 2 (CIC) are built");
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t ng = (size_t)nd * nd * nd;
  const float* g = grid;
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_GRID].ensure(sizeof(float) * ng));
    EXH_CUDA_TRY(cudaMemcpyAsync(c.buf[B_GRID].p, grid, sizeof(float) * ng, cudaMemcpyHostToDevice, st));
    g = c.buf[B_GRID].as<float>();
  }
  EXH_TRY(c.buf[B_HOSTIO2].ensure((sizeof(double) * 2 + sizeof(long long)) * Nk));
  double* oP = c.buf[B_HOSTIO2].as<double>();
  double* oK = oP + Nk;
  long long* oN = reinterpret_cast<long long*>(oK + Nk);
  EXH_TRY(power_spectrum(c, g, nd, L, window, Nk, k_min, k_max, oP, oK, oN, st));
  std::string tmp((sizeof(double) * 2 + sizeof(long long)) * Nk, '\0');
  EXH_CUDA_TRY(cudaMemcpyAsync(&tmp[0], oP, tmp.size(), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  const double* hP = reinterpret_cast<const double*>(tmp.data());
  const double* hK = hP + Nk;
  const long long* hN = reinterpret_cast<const long long*>(hK + Nk);
  for (int b = 0; b < Nk; b++) {
    P_out[b] = (float)hP[b];
    k_out[b] = (float)hK[b];
    count_out[b] = (int64_t)hN[b];
  }
  return EXH_OK;
}

}  // extern "C"
