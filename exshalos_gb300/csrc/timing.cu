// Event-based kernel-class timing (see timing.cuh).
#include <mutex>
#include <vector>

#include "exh_common.cuh"
#include "timing.cuh"

namespace exh {

namespace {
struct Rec {
  int cls;
  cudaEvent_t a, b;
  double bytes;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
thread_local cudaEvent_t t_open[KC_COUNT] = {};

cudaEvent_t take() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

bool timing_on() { return g_on; }

void timing_begin(int cls, cudaStream_t st) {
  std::lock_guard<std::mutex> g(g_mu);
  cudaEvent_t e = take();
  cudaEventRecord(e, st);
  t_open[cls] = e;
}

void timing_end(int cls, cudaStream_t st, double bytes) {
  std::lock_guard<std::mutex> g(g_mu);
  cudaEvent_t e = take();
  cudaEventRecord(e, st);
  g_recs.push_back({cls, t_open[cls], e, bytes});
  t_open[cls] = nullptr;
}

}  // namespace exh

using namespace exh;

extern "C" int exh_timing_enable(int on) {
  std::lock_guard<std::mutex> g(g_mu);
  g_on = on != 0;
  for (auto& r : g_recs) { g_pool.push_back(r.a); g_pool.push_back(r.b); }
  g_recs.clear();
  return EXH_OK;
}

// Per class: total milliseconds, launches and algorithmic bytes since the
// last enable.  Arrays of length n (<= number of classes); returns the
// number of classes written.
extern "C" int exh_timing_report(int n, double* ms, int64_t* launches, double* bytes) {
  std::lock_guard<std::mutex> g(g_mu);
  if (n > KC_COUNT) n = KC_COUNT;
  for (int i = 0; i < n; i++) { ms[i] = 0; launches[i] = 0; bytes[i] = 0; }
  for (auto& r : g_recs) {
    if (r.cls >= n) continue;
    cudaEventSynchronize(r.b);
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    ms[r.cls] += t;
    launches[r.cls] += 1;
    bytes[r.cls] += r.bytes;
  }
  return n;
}
