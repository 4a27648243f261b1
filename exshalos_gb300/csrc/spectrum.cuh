#pragma once
#include "ctx.cuh"

namespace exh {

struct BinParams {
  int Nk;
  float kn, kmin, dk, Lb, Normk;
  int window;
};

int cic_assign(Ctx& c, const float* pos_dev, int64_t np, int nd, float L, float* grid_dev, cudaStream_t st);
int power_spectrum(Ctx& c, const float* grid_dev, int nd, float L, int window, int Nk, float kmin, float kmax,
                   double* outP_dev, double* outK_dev, long long* outN_dev, cudaStream_t st);

}  // namespace exh
