#pragma once
#include "ctx.cuh"
#include "setup.h"

namespace exh {

void halo_state_release(Ctx& c);

// Gaussian field into `delta_dev` (float, x Normx), density_grid.c:71-217
int field_real(Ctx& c, const BoxParams& b, const float* K, const float* P, int Nk, int stream, int fixed,
               float phase, float* delta_dev, cudaStream_t st);

}  // namespace exh
