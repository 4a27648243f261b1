// Optional per-kernel-class timing with CUDA events recorded on the
// launching stream (enabled by exh_timing_enable).  Each record keeps the
// algorithmic bytes of the launch so that achieved bandwidth can be reported
// per class.
#pragma once
#include <cuda_runtime.h>

namespace exh {

enum KClass {
  KC_FFT_STRIDED = 0,   // x / y passes (incl. fused producers and consumers)
  KC_FFT_ROWS,          // z passes (real <-> half complex)
  KC_PEAKS,
  KC_SORT,
  KC_GROW,
  KC_MASS,
  KC_LPT_STENCIL,
  KC_HALO_DISP,
  KC_CIC,
  KC_BIN,
  KC_OTHER,
  KC_COUNT
};

bool timing_on();
void timing_begin(int cls, cudaStream_t st);
void timing_end(int cls, cudaStream_t st, double bytes);

struct KTimer {
  int cls;
  cudaStream_t st;
  double bytes;
  bool on;
  KTimer(int c, cudaStream_t s, double b) : cls(c), st(s), bytes(b), on(timing_on()) {
    if (on) timing_begin(cls, st);
  }
  ~KTimer() {
    if (on) timing_end(cls, st, bytes);
  }
};

}  // namespace exh
