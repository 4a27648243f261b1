// Batched realisations: many boxes of uneven size, each from its own Philox
// seed, each giving its halo catalogue and the shell-binned P(k) of the CIC
// grid of its halos (the chain of Generate_Halos_Box_from_Pk, mock.py:11-39 ->
// Compute_Density_Grid, simulation.py:9-26 -> Compute_Power_Spectrum,
// simulation.py:170-184, with the defaults of those calls).
//
// Scheduler: the realisations run on "lanes".  A lane is a library context
// (its own buffers and FFT plans) with its own non-blocking stream, driven by
// one host thread.  The halo finder's data-dependent loops (quicksort levels,
// growth rounds) read small counts back to the host; while one lane waits on
// such a read, the kernels of the other lanes keep the SMs busy, and the
// kernels of small boxes, which fill a fraction of the 152 SMs, run side by
// side.  Work is handed out largest box first from one shared counter
// (greedy list scheduling on the cell count), so the lanes finish together
// and each lane meets a new box size at most once per distinct size.
//
// Every realisation is computed by exactly the kernels of the one-box path,
// so its results do not depend on the lane count or on the assignment:
// lanes = 1 is the plain loop over realisations.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "ctx.cuh"

using namespace exh;

namespace {

int ensure_lanes(Ctx& c, int lanes) {
  while ((int)c.lane_ctx.size() < lanes) {
    exh_ctx* l = nullptr;
    EXH_TRY(exh_ctx_create(c.device, &l));
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      exh_ctx_destroy(l);
      cudaGetLastError();
      exh_set_error_msg("stream creation failed", __FILE__, __LINE__);
      return EXH_E_CUDA;
    }
    c.lane_ctx.push_back(l);
    c.lane_st.push_back(s);
  }
  return EXH_OK;
}

// one realisation on one lane: halos, CIC of the halo positions, P(k)
int run_item(exh_ctx* lane, cudaStream_t st, const float* k, const float* P, int Nk, exh_halo_params prm,
             const exh_batch_item& it, int Nk_pk, int64_t* nh, float* k_out, float* P_out, int64_t* n_out) {
  prm.ndx = prm.ndy = prm.ndz = it.nd;
  prm.seed = it.seed;
  EXH_TRY(exh_halos_box_from_pk(lane, k, P, Nk, &prm, nh, st));
  Ctx& c = lane->c;
  const int nd = it.nd;
  const float L = prm.Lc * (float)nd;
  EXH_TRY(c.buf[B_GRID].ensure(sizeof(float) * (size_t)nd * nd * nd));
  float* grid = c.buf[B_GRID].as<float>();
  EXH_TRY(exh_grid_compute(lane, c.halos.posh, *nh, nd, L, 2, 1, grid, EXH_MEM_DEVICE, st));
  const float kmin = (float)(2.0 * M_PI / L), kmax = (float)(M_PI * nd / L);
  return exh_power_compute(lane, grid, nd, L, 2, Nk_pk, kmin, kmax, k_out, P_out, n_out, EXH_MEM_DEVICE, st);
}

}  // namespace

extern "C" int exh_batch_run(exh_ctx* ctx, const float* k, const float* P, int Nk, const exh_halo_params* base,
                             const exh_batch_item* items, int n, int Nk_pk, int lanes, int64_t* nh_out,
                             float* k_out, float* P_out, int64_t* count_out, int32_t* status_out) {
  if (!ctx || !k || !P || !base || (n > 0 && (!items || !nh_out || !k_out || !P_out || !count_out))) {
    exh_set_error_msg("null argument", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  if (n < 0 || lanes < 1 || lanes > 64 || Nk_pk < 1 || Nk_pk > 4096) {
    exh_set_error_msg("need n >= 0, 1 <= lanes <= 64 and 1 <= Nk_pk <= 4096", __FILE__, __LINE__);
    return EXH_E_INVALID;
  }
  for (int i = 0; i < n; i++) {
    if (items[i].nd < 8 || items[i].nd > 1024 || (items[i].nd & 1)) {
      exh_set_error_msg("each box needs an even nd in [8, 1024]", __FILE__, __LINE__);
      return EXH_E_INVALID;
    }
  }
  if (n == 0) return EXH_OK;
  Ctx& c = ctx->c;
  EXH_CUDA_TRY(cudaSetDevice(c.device));
  lanes = std::min(lanes, n);
  EXH_TRY(ensure_lanes(c, lanes));
  // largest boxes first; ties keep the caller's order
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return items[a].nd > items[b].nd; });
  std::atomic<int> next{0};
  std::atomic<int> failed{0};
  std::vector<int> status(lanes, EXH_OK);
  std::vector<std::string> msg(lanes);
  auto worker = [&](int w) {
    exh_ctx* lane = c.lane_ctx[w];
    cudaStream_t st = c.lane_st[w];
    if (cudaSetDevice(c.device) != cudaSuccess) {
      status[w] = EXH_E_CUDA;
      msg[w] = "cudaSetDevice failed";
      failed.store(1);
      return;
    }
    for (;;) {
      if (failed.load()) return;
      const int j = next.fetch_add(1);
      if (j >= n) return;
      const int i = order[j];
      const int s = run_item(lane, st, k, P, Nk, *base, items[i], Nk_pk, &nh_out[i], k_out + (size_t)i * Nk_pk,
                             P_out + (size_t)i * Nk_pk, count_out + (size_t)i * Nk_pk);
      if (status_out) status_out[i] = s;
      // with a status array, a realisation outside the tables (EXH_E_RANGE)
      // is reported there and the batch goes on; anything else stops it
      if (s == EXH_E_RANGE && status_out) {
        nh_out[i] = -1;
        continue;
      }
      if (s != EXH_OK) {
        status[w] = s;
        msg[w] = std::string("realisation ") + std::to_string(i) + ": " + exh_last_error();
        failed.store(1);
        return;
      }
    }
  };
  if (lanes == 1) {
    worker(0);
  } else {
    std::vector<std::thread> th;
    th.reserve(lanes);
    for (int w = 0; w < lanes; w++) th.emplace_back(worker, w);
    for (auto& t : th) t.join();
  }
  for (int w = 0; w < lanes; w++) {
    if (status[w] != EXH_OK) {
      exh_set_error_msg(msg[w].c_str(), __FILE__, __LINE__);
      return status[w];
    }
  }
  return EXH_OK;
}
