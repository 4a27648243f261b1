// Gaussian field: modes (Philox, or the reference's taus stream drawn
// beforehand) generated inside the first pass of the inverse FFT, scaled by
// Normx in the last pass (density_grid.c:71-217).
#include <cmath>
#include <string>
#include <vector>

#include "ctx.cuh"
#include "fft4.cuh"
#include "field.cuh"
#include "lpt.cuh"
#include "pipeline.cuh"

namespace exh {

int upload_amplitudes(Ctx& c, const BoxParams& b, const float* K, const float* P, int Nk, float** A_dev,
                      cudaStream_t st) {
  std::string key;
  key.append(reinterpret_cast<const char*>(b.nd), sizeof(b.nd));
  key.append(reinterpret_cast<const char*>(&b.Lc), sizeof(float));
  key.append(reinterpret_cast<const char*>(K), sizeof(float) * Nk);
  key.append(reinterpret_cast<const char*>(P), sizeof(float) * Nk);
  if (key == c.amp_key && c.buf[B_TAB].p) {
    *A_dev = c.buf[B_TAB].as<float>();
    return EXH_OK;
  }
  c.amp_key.clear();
  std::vector<float> A;
  int s = amplitude_table(b, K, P, Nk, A);
  if (s == EXH_E_UNSUPPORTED) {
    exh_set_error_msg("the field is built for cubic boxes (ndx == ndy == ndz)", __FILE__, __LINE__);
    return s;
  }
  if (s != EXH_OK) {
    exh_set_error_msg("P(k) table does not cover the box's wave numbers", __FILE__, __LINE__);
    return s;
  }
  EXH_TRY(c.buf[B_TAB].ensure(sizeof(float) * A.size()));
  EXH_CUDA_TRY(cudaMemcpyAsync(c.buf[B_TAB].p, A.data(), sizeof(float) * A.size(), cudaMemcpyHostToDevice, st));
  // the host vector dies here: wait for the copy
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  *A_dev = c.buf[B_TAB].as<float>();
  c.amp_key = key;
  return EXH_OK;
}

FieldModes make_modes(const BoxParams& b, const float* A_dev, int fixed, float phase) {
  FieldModes m;
  m.n0 = b.nd[0]; m.n1 = b.nd[1]; m.n2 = b.nd[2]; m.nc = b.nz2;
  m.seed = (uint32_t)b.seed;
  m.fixed = fixed;
  m.use_phase = phase != 0.0f;
  m.cph = (float)std::cos((double)phase);
  m.sph = (float)std::sin((double)phase);
  m.A = A_dev;
  m.draws = nullptr;
  return m;
}

int make_field_modes(Ctx& c, const BoxParams& b, const float* A_dev, int stream, int fixed, float phase,
                     cudaStream_t st, FieldModes* out) {
  *out = make_modes(b, A_dev, fixed, phase);
  if (stream == EXH_FIELD_TAUS) {
    const float* d = nullptr;
    EXH_TRY(taus_field_draws(c, b, fixed, st, &d));
    out->draws = d;
  }
  return EXH_OK;
}

int field_real(Ctx& c, const BoxParams& b, const float* K, const float* P, int Nk, int stream, int fixed,
               float phase, float* delta_dev, cudaStream_t st) {
  FFTPlan3D* p;
  EXH_TRY(c.get_plan(b.nd[0], b.nd[1], b.nd[2], &p));
  float* A_dev = nullptr;
  EXH_TRY(upload_amplitudes(c, b, K, P, Nk, &A_dev, st));
  const size_t nk = (size_t)b.nd[0] * b.nd[1] * p->nc;
  EXH_TRY(c.buf[B_WORK].ensure(sizeof(float2) * nk));
  float2* work = c.buf[B_WORK].as<float2>();
  FieldGen gen;
  EXH_TRY(make_field_modes(c, b, A_dev, stream, fixed, phase, st, &gen.m));
  EXH_CUDA_TRY(fft_c2r_3d(*p, gen, work, RealPairStore{delta_dev, b.nd[2], b.Normx}, st));
  return EXH_OK;
}

}  // namespace exh
