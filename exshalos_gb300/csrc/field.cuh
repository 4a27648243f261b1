// Gaussian-field synthesis as a generator for the first pass of the inverse
// FFT (Compute_Den, src/exshalos/density_grid.c:71-217).
//
// Two random streams:
//  * Philox (EXH_FIELD_PHILOX): each independent half-complex mode draws one
//    Philox4x32-10 block keyed by (seed, mode index);
//  * the reference's own (EXH_FIELD_TAUS): the deviates of its sequential
//    gsl_rng_taus stream, generated beforehand in loop order
//    (taus_field.cu), which a mode reads at the index its position in the
//    reference's loop gives (taus_draw_index).
// In both, the Hermitian partners on the kz = 0 and kz = nz/2 planes come
// from their source mode, conjugated, following the four copy rules of
// density_grid.c:109-150.  The amplitude sqrt(P(k)/2) is read from a table
// indexed by the integer |n|^2 of the mode.  Nothing is stored in k space:
// consumers regenerate the modes they need.
#pragma once
#include "exh_common.cuh"
#include "taus_index.h"

namespace exh {

constexpr uint32_t PHILOX_KEY1 = 0x45584853u;

__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                              uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct FieldModes {
  int n0, n1, n2, nc;
  uint32_t seed;
  int fixed;
  float cph, sph;              // cos/sin of the constant phase (0, 1 when unused)
  int use_phase;
  const float* __restrict__ A; // sqrt(P/2) by |n|^2
  // taus stream: the field's deviates (phases with `fixed`) in draw order;
  // nullptr for the Philox stream
  const float* __restrict__ draws;

  // mode (i, j, k) of the half-complex grid
  __device__ __forceinline__ float2 mode(int i, int j, int k) const {
    int si = i, sj = j;
    bool conj = false;
    if ((k == 0 || k == n2 / 2) && (i > n0 / 2 || j > n1 / 2)) {
      if (i > n0 / 2 && j > n1 / 2) { si = n0 - i; sj = n1 - j; conj = true; }
      else if (i == 0 || i == n0 / 2) { sj = n1 - j; conj = true; }
      else if (j == 0 || j == n1 / 2) { si = n0 - i; conj = true; }
      else if (i > n0 / 2 && j < n1 / 2) { si = n0 - i; sj = n1 - j; conj = true; }
    }
    const int ii = si < n0 / 2 ? si : si - n0;
    const int jj = sj < n1 / 2 ? sj : sj - n1;
    const int kk = (k == n2 / 2) ? n2 / 2 : k;
    const int q2 = ii * ii + jj * jj + kk * kk;
    const float a = A[q2];
    if (draws) return taus_mode(si, sj, k, a, conj);
    const uint64_t ind = ((uint64_t)si * n1 + sj) * nc + k;
    uint32_t o[4];
    philox4x32_10((uint32_t)ind, (uint32_t)(ind >> 32), 0u, 0u, seed, PHILOX_KEY1, o);
    const float u1 = ((float)(o[0] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = (float)(o[1] >> 8) * (1.0f / 16777216.0f);
    float re, im;
    const bool selfc = (si == 0 || si == n0 / 2) && (sj == 0 || sj == n1 / 2) && (k == 0 || k == n2 / 2);
    if (fixed) {
      if (selfc) { re = 1.41421356237309515f * a; im = 0.f; }
      else {
        float s, c;
        sincospif(2.0f * (float)(o[2] >> 8) * (1.0f / 16777216.0f), &s, &c);
        re = a * c; im = a * s;
      }
    } else {
      const float rad = sqrtf(-2.0f * logf(u1));
      float s, c;
      sincospif(2.0f * u2, &s, &c);
      if (selfc) { re = 1.41421356237309515f * a * (rad * c); im = 0.f; }
      else { re = a * (rad * c); im = a * (rad * s); }
    }
    if (use_phase) {   // density_grid.c:189-192, second line reads the rotated real part
      const float r0 = re * cph - im * sph;
      im = r0 * sph + im * cph;
      re = r0;
    }
    return conj ? make_float2(re, -im) : make_float2(re, im);
  }

  // the reference's arithmetic (density_grid.c:169-186): A times the float
  // deviate in float; the self-conjugate modes sqrt(2.0) A g in double;
  // `fixed`: A cos(theta), A sin(theta) in double from the float phase
  __device__ __forceinline__ float2 taus_mode(int si, int sj, int k, float a, bool conj) const {
    const bool selfc = (si == 0 || si == n0 / 2) && (sj == 0 || sj == n1 / 2) && (k == 0 || k == n2 / 2);
    const long long d = taus_draw_index(si, sj, k, n0, n1, n2, fixed);
    float re, im;
    if (fixed) {
      if (selfc) { re = __double2float_rn(__dmul_rn(1.4142135623730951, (double)a)); im = 0.f; }
      else {
        double sn, cs;
        sincos((double)draws[d], &sn, &cs);
        re = __double2float_rn(__dmul_rn((double)a, cs));
        im = __double2float_rn(__dmul_rn((double)a, sn));
      }
    } else if (selfc) {
      re = __double2float_rn(__dmul_rn(__dmul_rn(1.4142135623730951, (double)a), (double)draws[d]));
      im = 0.f;
    } else {
      re = __fmul_rn(a, draws[d]);
      im = __fmul_rn(a, draws[d + 1]);
    }
    if (use_phase) {
      const float r0 = re * cph - im * sph;
      im = r0 * sph + im * cph;
      re = r0;
    }
    return conj ? make_float2(re, -im) : make_float2(re, im);
  }
};

// Source functor of the x pass: (o = 0, e = i, inner = j * nc + k)
struct FieldGen {
  static constexpr int io_bytes = 0;
  FieldModes m;
  __device__ __forceinline__ float2 operator()(int, int e, int inner) const {
    return m.mode(e, inner / m.nc, inner % m.nc);
  }
};

}  // namespace exh
