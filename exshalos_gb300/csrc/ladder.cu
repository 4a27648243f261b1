// FFT top-hat smoothing ladder and per-cell first-crossing map.
//
// For n_radii radii R_i log-spaced from one cell to R_max, the field is
// smoothed with the top-hat window W(kR) = 3 (sin x - x cos x) / x^3
// (exshalos_h.c:35-40) by one inverse FFT per radius, and each cell records
// the largest radius at which the smoothed density reaches the excursion-set
// barrier B(sigma^2(R)) (find_halos.c:4-44, 200-212): the first crossing when
// the ladder is walked from large to small scales.  255 = never crossed.
//
// The Fourier modes are generated once (the same Philox modes as the field)
// and read by the first pass of every radius; the barrier test and the map
// update run in the epilogue of the last pass, so no smoothed field is ever
// stored.
#include <cmath>
#include <vector>

#include "ctx.cuh"
#include "fft4.cuh"
#include "field.cuh"
#include "lpt.cuh"
#include "setup.h"

namespace exh {

__global__ void k_store_modes(FieldModes m, float2* __restrict__ out) {
  const size_t nk = (size_t)m.n0 * m.n1 * m.nc;
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; t < nk; t += stride) {
    const int k = (int)(t % m.nc);
    const size_t r = t / m.nc;
    out[t] = m.mode((int)(r / m.n1), (int)(r % m.n1), k);
  }
}

__device__ __forceinline__ float tophat(float x) {
  if (x < 1e-2f) {                       // series: 1 - x^2/10 + x^4/280
    const float x2 = x * x;
    return 1.f - x2 * (0.1f - x2 * (1.f / 280.f));
  }
  float s, c;
  sincosf(x, &s, &c);
  return 3.f * (s - x * c) / (x * x * x);
}

// x-pass source: stored modes times W(|k| R)
struct LadderGen {
  static constexpr int io_bytes = 8;
  const float2* __restrict__ dk;
  int n0, n1, n2, nc;
  float kl0, kl1, kl2, R;
  __device__ __forceinline__ float2 operator()(int, int e, int inner) const {
    const int j = inner / nc, k = inner % nc;
    const float kx = (float)((2 * e < n0) ? e : e - n0) * kl0;
    const float ky = (float)((2 * j < n1) ? j : j - n1) * kl1;
    const float kz = (float)((k == n2 / 2) ? -(n2 / 2) : k) * kl2;
    const float w = tophat(sqrtf(kx * kx + ky * ky + kz * kz) * R);
    const float2 v = dk[(size_t)e * inner_size() + inner];
    return make_float2(v.x * w, v.y * w);
  }
  __device__ __forceinline__ size_t inner_size() const { return (size_t)n1 * nc; }
};

// z-pass destination: barrier test, first crossing kept
struct CrossStore {
  static constexpr int io_bytes = 4;     // two u8 reads and writes per pair
  unsigned char* __restrict__ cross;
  int N;
  float normx, B;
  int r;
  __device__ __forceinline__ void operator()(size_t row, int m, float2 v) const {
    unsigned char* c = cross + row * N + 2 * m;
    const unsigned char c0 = c[0], c1 = c[1];
    if (c0 == 255 && v.x * normx >= B) c[0] = (unsigned char)r;
    if (c1 == 255 && v.y * normx >= B) c[1] = (unsigned char)r;
  }
};

int smoothing_ladder(Ctx& c, const BoxParams& b, const FieldModes& modes, int n_radii, const float* R,
                     const float* B, unsigned char* cross, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
  const size_t nk = (size_t)b.nd[0] * b.nd[1] * p->nc;
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  EXH_TRY(c.buf[B_LADDER].ensure(sizeof(float2) * nk));
  float2* work = c.buf[B_WORK].as<float2>();
  float2* dk = c.buf[B_LADDER].as<float2>();
  {
    KTimer kt(KC_OTHER, st, 8.0 * nk);
    k_store_modes<<<EXH_NUM_SMS * 16, 256, 0, st>>>(modes, dk);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  EXH_CUDA_TRY(cudaMemsetAsync(cross, 255, b.ng, st));
  for (int i = n_radii - 1; i >= 0; i--) {       // large scales first
    LadderGen gen{dk, b.nd[0], b.nd[1], b.nd[2], p->nc, b.kl[0], b.kl[1], b.kl[2], R[i]};
    CrossStore cs{cross, b.nd[2], b.Normx, B[i], i};
    EXH_CUDA_TRY(fft_c2r_3d(*p, gen, work, cs, st));
  }
  return EXH_OK;
}

}  // namespace exh

using namespace exh;

extern "C" int exh_smoothing_ladder(exh_ctx* ctx, const float* k, const float* P, int Nk, const exh_halo_params* prm,
                                    int n_radii, float R_max, uint8_t* cross, float* radii_out, float* barrier_out,
                                    int mem, void* stream) {
  if (!ctx || !k || !P || !prm || !cross) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  BoxParams b;
  EXH_TRY(setup_box(&b, prm->ndx, prm->ndy, prm->ndz, prm->Lc, prm->Om0, prm->redshift, prm->dc, prm->Nmin, prm->a,
                    prm->beta, prm->alpha, prm->seed));
  std::vector<float> R, B;
  if (ladder_tables(b, k, P, Nk, n_radii, R_max, R, B) != EXH_OK) {
    exh_set_error_msg("ladder needs 1..255 radii and R_max >= Lc", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  float* A_dev = nullptr;
  EXH_TRY(upload_amplitudes(c, b, k, P, Nk, &A_dev, st));
  const FieldModes modes = make_modes(b, A_dev, prm->fixed, prm->phase);
  unsigned char* out = reinterpret_cast<unsigned char*>(cross);
  if (mem == EXH_MEM_HOST) {
    EXH_TRY(c.buf[B_CROSS].ensure(b.ng));
    out = c.buf[B_CROSS].as<unsigned char>();
  }
  EXH_TRY(smoothing_ladder(c, b, modes, n_radii, R.data(), B.data(), out, st));
  if (mem == EXH_MEM_HOST) EXH_CUDA_TRY(cudaMemcpyAsync(cross, out, b.ng, cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  for (int i = 0; i < n_radii; i++) {
    if (radii_out) radii_out[i] = R[i];
    if (barrier_out) barrier_out[i] = B[i];
  }
  return EXH_OK;
}
