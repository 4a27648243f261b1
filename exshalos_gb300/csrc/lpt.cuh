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
int upload_amplitudes(Ctx& c, const BoxParams& b, const float* K, const float* P, int Nk, float** A_dev,
                      cudaStream_t st);

}  // namespace exh
