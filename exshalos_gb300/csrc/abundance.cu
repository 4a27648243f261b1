// Differential halo abundance: abundance_compute (src/spectrum/spectrum.c:535-600)
// -> Measure_Abundance (src/spectrum/abundance.c:4-36).  Log-mass bins of
// width dlnM = (ln Mmax - ln Mmin) / Nm (a float, as the reference stores
// it); per bin the count, the mean mass (summed in FP64) and
// dn = N / V / dlnM, dn_err = sqrt(N) / V / dlnM.
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.cuh"

namespace exh {
namespace {

constexpr int AB_T = 256;
constexpr int AB_MAX_BINS = 4096;

__global__ void k_mass_range(const float* __restrict__ M, int64_t n, unsigned* __restrict__ mm) {
  // min and max of positive floats through their ordered bit patterns
  unsigned lo = 0xFFFFFFFFu, hi = 0u;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned u = __float_as_uint(M[i]);
    lo = min(lo, u);
    hi = max(hi, u);
  }
  atomicMin(&mm[0], lo);
  atomicMax(&mm[1], hi);
}

__global__ void __launch_bounds__(AB_T)
k_abundance(const float* __restrict__ M, int64_t n, double lnMmin, double dlnM, int Nm,
            unsigned long long* __restrict__ cnt, double* __restrict__ msum) {
  extern __shared__ unsigned char sm_raw[];
  double* hs = reinterpret_cast<double*>(sm_raw);
  unsigned* hc = reinterpret_cast<unsigned*>(hs + Nm);
  for (int b = threadIdx.x; b < Nm; b += blockDim.x) { hs[b] = 0.0; hc[b] = 0u; }
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float m = M[i];
    const int ind = (int)floor((log((double)m) - lnMmin) / dlnM);
    if (ind > 0 && ind < Nm) {            // abundance.c:22: bin 0 is left out, as there
      atomicAdd(&hc[ind], 1u);
      atomicAdd(&hs[ind], (double)m);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < Nm; b += blockDim.x) {
    if (hc[b]) {
      atomicAdd(&cnt[b], (unsigned long long)hc[b]);
      atomicAdd(&msum[b], hs[b]);
    }
  }
}

}  // namespace
}  // namespace exh

using namespace exh;

extern "C" int exh_abundance_compute(exh_ctx* ctx, const float* Mh, int64_t nh, float Mmin, float Mmax, int Nm,
                                     float Lc, int ndx, int ndy, int ndz, float* Mmean, float* dn, float* dn_err,
                                     int mem, void* stream) {
  if (!ctx || (nh > 0 && !Mh) || !Mmean || !dn || !dn_err) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (nh < 0 || Nm < 1 || Nm > AB_MAX_BINS || !(Lc > 0.f) || ndx < 1 || ndy < 1 || ndz < 1) {
    exh_set_error_msg("need nh >= 0, 1 <= Nm <= 4096, Lc > 0 and positive grid sizes", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = (cudaStream_t)stream;
  const float* d = Mh;
  if (mem == EXH_MEM_HOST && nh > 0) {
    EXH_TRY(c.buf[B_HOSTIO].ensure(sizeof(float) * (size_t)nh));
    EXH_CUDA_TRY(cudaMemcpyAsync(c.buf[B_HOSTIO].p, Mh, sizeof(float) * (size_t)nh, cudaMemcpyHostToDevice, st));
    d = c.buf[B_HOSTIO].as<float>();
  }
  EXH_TRY(c.buf[B_SCRATCH].ensure(64 + (sizeof(unsigned long long) + sizeof(double)) * (size_t)Nm));
  unsigned* mm = c.buf[B_SCRATCH].as<unsigned>();
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(c.buf[B_SCRATCH].as<char>() + 64);
  double* msum = reinterpret_cast<double*>(cnt + Nm);
  const unsigned nb = (unsigned)std::min<int64_t>(std::max<int64_t>((nh + AB_T - 1) / AB_T, 1), EXH_NUM_SMS * 4);
  // spectrum.c:566-578: the range from the masses, widened by 1e-4
  if (Mmin < 0.f || Mmax < 0.f) {
    const unsigned init[2] = {0xFFFFFFFFu, 0u};
    EXH_TRY(upload_small(mm, init, sizeof(init), st));
    if (nh > 0) {
      k_mass_range<<<nb, AB_T, 0, st>>>(d, nh, mm);
      count_launch(1);
      EXH_CUDA_TRY(cudaGetLastError());
    }
    unsigned h[2];
    EXH_CUDA_TRY(cudaMemcpyAsync(h, mm, sizeof(h), cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    float lo, hi;
    std::memcpy(&lo, &h[0], 4);
    std::memcpy(&hi, &h[1], 4);
    if (Mmin < 0.f) Mmin = (float)((nh > 0 ? std::min(lo, 1e20f) : 1e20f) * 0.9999);
    if (Mmax < 0.f) Mmax = (float)((nh > 0 ? hi : Mmax) * 1.0001);
  }
  if (!(Mmin > 0.f) || !(Mmax > Mmin)) {
    exh_set_error_msg("the mass range must satisfy 0 < Mmin < Mmax", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  const float dlnM = (float)((std::log((double)Mmax) - std::log((double)Mmin)) / Nm);     // abundance.c:10
  EXH_CUDA_TRY(cudaMemsetAsync(cnt, 0, (sizeof(unsigned long long) + sizeof(double)) * (size_t)Nm, st));
  if (nh > 0) {
    const size_t sm = (sizeof(double) + sizeof(unsigned)) * (size_t)Nm + 16;
    if (sm > 48 * 1024) EXH_CUDA_TRY(set_smem(k_abundance, sm));
    k_abundance<<<nb, AB_T, sm, st>>>(d, nh, std::log((double)Mmin), (double)dlnM, Nm, cnt, msum);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  std::vector<unsigned long long> hc(Nm);
  std::vector<double> hs(Nm);
  EXH_CUDA_TRY(cudaMemcpyAsync(hc.data(), cnt, sizeof(unsigned long long) * Nm, cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaMemcpyAsync(hs.data(), msum, sizeof(double) * Nm, cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  const float V = (Lc * ndx) * (Lc * ndy) * (Lc * ndz);     // Lx*Ly*Lz in float
  for (int i = 0; i < Nm; i++) {
    const int N = (int)hc[i];
    Mmean[i] = N > 0 ? (float)(hs[i] / N) : 0.f;
    dn[i] = (float)N / V / dlnM;
    dn_err[i] = (float)(std::sqrt((double)N) / V / dlnM);
  }
  return EXH_OK;
}
