// The adaptive schedule of the stationary mixed-precision loop, shared by
// the device-side loop controller and the host loop (and plain C++, for the
// tests).
#pragma once

#if defined(__CUDACC__)
#define GBMG_HOST_DEVICE __host__ __device__
#else
#define GBMG_HOST_DEVICE
#endif

namespace gbmg {

// Cycles the next correction needs, predicted from the last one: it took the
// relative residual from prev to rel in s cycles, so a cycle multiplies it by
// r = (rel/prev)^(1/s); the answer is the smallest k < step_max with
// rel r^k < tol, i.e. rel^s (rel/prev)^k < tol^s (products only, so the host
// and the device decide alike), else step_max.
GBMG_HOST_DEVICE inline int tail_cycles(double rel, double prev, double tol, int s,
                                           int step_max) {
  const double ratio = rel / prev;
  double q = 1.0, t = 1.0;
  for (int i = 0; i < s; ++i) {
    q *= rel;
    t *= tol;
  }
  for (int k = 1; k < step_max; ++k) {
    q *= ratio;
    if (q < t) return k;
  }
  return step_max;
}

}  // namespace gbmg
