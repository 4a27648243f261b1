// FFT plans and the plain 3-D transforms of the C ABI.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "ctx.cuh"
#include "fft4.cuh"

namespace exh {

cudaError_t smem_raise(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> limit;     // (device, kernel) -> limit set
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = limit[std::make_pair(dev, kernel)];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

RadixPlan make_radix_plan(int n) {
  RadixPlan p{};
  p.n = n;
  p.nst = 0;
  int m = n;
  while (m % 8 == 0 && p.nst < 12) { p.r[p.nst++] = 8; m /= 8; }
  while (m % 4 == 0 && p.nst < 12) { p.r[p.nst++] = 4; m /= 4; }
  while (m % 2 == 0 && p.nst < 12) { p.r[p.nst++] = 2; m /= 2; }
  while (m % 3 == 0 && p.nst < 12) { p.r[p.nst++] = 3; m /= 3; }
  if (m != 1) p.nst = -1;   // a prime factor other than 2 or 3
  return p;
}

static int upload_twiddles(int n, float2** out) {
  std::vector<float2> h(n);
  for (int m = 0; m < n; m++) {
    double s, c;
    sincospi(2.0 * (double)m / (double)n, &s, &c);
    h[m] = make_float2((float)c, (float)s);
  }
  if (cudaMalloc(out, sizeof(float2) * n) != cudaSuccess) {
    cudaGetLastError();
    return EXH_E_NOMEM;
  }
  EXH_CUDA_TRY(cudaMemcpy(*out, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  return EXH_OK;
}

int fft_plan_create(FFTPlan3D* p, int nx, int ny, int nz) {
  if (nx < 2 || ny < 2 || nz < 4 || (nz & 1)) {
    exh_set_error_msg("FFT sizes must be >= 2 with an even last axis", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  p->nx = nx; p->ny = ny; p->nz = nz; p->nc = nz / 2 + 1; p->M = nz / 2;
  p->px = make_radix_plan(nx);
  p->py = make_radix_plan(ny);
  p->pm = make_radix_plan(p->M);
  if (p->px.nst < 0 || p->py.nst < 0 || p->pm.nst < 0 || nx > 1024 || ny > 1024 || p->M > 512) {
    exh_set_error_msg("FFT sizes must be 2^a 3^b with nx, ny <= 1024 and nz <= 1024", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  EXH_TRY(upload_twiddles(nx, &p->twx));
  EXH_TRY(upload_twiddles(ny, &p->twy));
  EXH_TRY(upload_twiddles(p->M, &p->twm));
  EXH_TRY(upload_twiddles(nz, &p->twn));
  return EXH_OK;
}

void fft_plan_destroy(FFTPlan3D* p) {
  cudaFree(p->twx); cudaFree(p->twy); cudaFree(p->twm); cudaFree(p->twn);
  p->twx = p->twy = p->twm = p->twn = nullptr;
}

int Ctx::capture_stream(cudaStream_t* out) {
  if (!capture) EXH_CUDA_TRY(cudaStreamCreateWithFlags(&capture, cudaStreamNonBlocking));
  *out = capture;
  return EXH_OK;
}

int build_while_graph(Ctx& c, const std::function<int(cudaStream_t, cudaGraphConditionalHandle)>& body,
                      cudaGraph_t* src_out, cudaGraphExec_t* exec_out) {
  cudaStream_t cs;
  EXH_TRY(c.capture_stream(&cs));
  cudaGraph_t g = nullptr;
  EXH_CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np{};
  cudaGraphNode_t node;
  if (e == cudaSuccess) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  }
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                          cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    exh_set_error_msg(cudaGetErrorString(e), __FILE__, __LINE__);
    return EXH_E_CUDA;
  }
  const int bs = body(cs, h);
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(cs, &captured);
  cudaGraphExec_t ex = nullptr;
  if (bs == EXH_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
  if (bs != EXH_OK || e != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    if (bs != EXH_OK) return bs;
    exh_set_error_msg(cudaGetErrorString(e), __FILE__, __LINE__);
    return EXH_E_CUDA;
  }
  *src_out = g;
  *exec_out = ex;
  return EXH_OK;
}

int Ctx::side_stream(cudaStream_t* out) {
  if (!side) {
    EXH_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    EXH_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    EXH_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  }
  *out = side;
  return EXH_OK;
}

namespace {
struct SmallBlob {
  unsigned char b[UPLOAD_SMALL_MAX];
};
__global__ void k_upload_small(unsigned char* __restrict__ dst, SmallBlob blob, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = blob.b[i];
}
}  // namespace

int upload_small(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return EXH_OK;
  if (!dst || !src || bytes > UPLOAD_SMALL_MAX) return EXH_E_INVALID;
  SmallBlob blob;
  std::memcpy(blob.b, src, bytes);
  k_upload_small<<<1, 64, 0, st>>>(reinterpret_cast<unsigned char*>(dst), blob, (int)bytes);
  count_launch(1);
  return cudaGetLastError() == cudaSuccess ? EXH_OK : EXH_E_CUDA;
}

int Ctx::fork_stream(cudaStream_t st, cudaStream_t* out) {
  EXH_TRY(side_stream(out));
  if (timing_on()) *out = st;
  return EXH_OK;
}

int Ctx::get_plan(int nx, int ny, int nz, FFTPlan3D** out) {
  auto key = std::make_tuple(nx, ny, nz);
  auto it = plans.find(key);
  if (it == plans.end()) {
    FFTPlan3D p;
    int s = fft_plan_create(&p, nx, ny, nz);
    if (s != EXH_OK) return s;
    it = plans.emplace(key, p).first;
  }
  *out = &it->second;
  return EXH_OK;
}

}  // namespace exh

using namespace exh;

extern "C" int exh_fft_r2c_3d(exh_ctx* ctx, int nx, int ny, int nz, const float* in, float* out, void* stream) {
  if (!ctx || !in || !out) return EXH_E_INVALID;
  FFTPlan3D* p;
  EXH_TRY(ctx->c.get_plan(nx, ny, nz, &p));
  float2* work = reinterpret_cast<float2*>(out);
  cudaStream_t st = (cudaStream_t)stream;
  EXH_CUDA_TRY(fft_r2c_3d(*p, RealPairLoad{in, nz}, work, CplxStore{work, nx, ny * p->nc}, st));
  return EXH_OK;
}

extern "C" int exh_fft_c2r_3d(exh_ctx* ctx, int nx, int ny, int nz, float* in, float* out, void* stream) {
  if (!ctx || !in || !out) return EXH_E_INVALID;
  FFTPlan3D* p;
  EXH_TRY(ctx->c.get_plan(nx, ny, nz, &p));
  float2* work = reinterpret_cast<float2*>(in);
  cudaStream_t st = (cudaStream_t)stream;
  EXH_CUDA_TRY(fft_c2r_3d(*p, CplxLoad{work, nx, ny * p->nc}, work, RealPairStore{out, nz, 1.f}, st));
  return EXH_OK;
}
