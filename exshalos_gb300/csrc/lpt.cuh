#pragma once
#include "ctx.cuh"
#include "field.cuh"
#include "halos.cuh"
#include "setup.h"

namespace exh {

struct HaloOut {
  float* posh;
  float* velh;     // may be null
  float Lc;
  float L[3];
  double f1, f2;   // velocity factors of the first- and second-order terms
};

// S (planes [3][ng]) = first (+ second) order displacement; V (optional) the
// matching velocities; phi1, phi2 are the potentials (work arrays)
int lpt_run(Ctx& c, const BoxParams& b, const FieldModes& modes, float k_smooth, bool do2, float* S, float* V,
            float* phi1, float* phi2, cudaStream_t st);
// the same from a given real field delta (device): delta_k = Normk r2c(delta)
int lpt_run_grid(Ctx& c, const BoxParams& b, const float* delta, float k_smooth, bool do2, float* S, float* V,
                 float* phi1, float* phi2, cudaStream_t st);
// particle arrays [ng][3] -> planes [3][ng]
int aos_to_planes(const float* in, size_t ng, float* out, cudaStream_t st);
HaloOut make_halo_out(const BoxParams& b, float* posh, float* velh);
int halo_displacements(Ctx& c, const BoxParams& b, const HaloDev& h, const ShellTable& t, const float* S,
                       const float* V, const HaloOut& o, cudaStream_t st);
int particles(const BoxParams& b, const float* S, const float* V, const HaloOut& o, float* pos, float* vel,
              cudaStream_t st);
FieldModes make_modes(const BoxParams& b, const float* A_dev, int fixed, float phase);
// the modes of field stream `stream` (EXH_FIELD_PHILOX or EXH_FIELD_TAUS;
// the taus stream's draws are generated on `st` first, taus_field.cu)
int make_field_modes(Ctx& c, const BoxParams& b, const float* A_dev, int stream, int fixed, float phase,
                     cudaStream_t st, FieldModes* out);
// the draws of the reference's taus stream for box b and its seed into
// context memory (*out): deviates, or with `fixed` phases, in draw order
// (or a copy of another context's draws of the same box and seed, when that
// context offers them)
int taus_field_draws(Ctx& c, const BoxParams& b, int fixed, cudaStream_t st, const float** out);
// withdraw c's offered draws and wait for the copies taken from them (before
// c's buffers are freed)
void taus_offer_release(Ctx& c);
// after the stream of the last taus_field_draws has been synchronised: did
// its stream hold every draw (EXH_E_RANGE if not)
int taus_verify(Ctx& c);
int upload_amplitudes(Ctx& c, const BoxParams& b, const float* K, const float* P, int Nk, float** A_dev,
                      cudaStream_t st);

}  // namespace exh
