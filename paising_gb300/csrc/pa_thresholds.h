// pa_thresholds.h -- per-temperature acceptance thresholds, shared by the
// host (fixed schedules, computed with the host's exp like the reference) and
// the adaptive-step kernel (schedules chosen on the device, device exp).
#pragma once

#include <cmath>
#include <cstdint>

#include "pa_state.h"

namespace pa {

// Integer thresholds of one temperature (kThrPerStep words):
//   [0..9]  SSC Boltzmann table boltz[idxT0 + 2 idxT1] = min(1, exp(-2 s sum_nn beta))
//           (PAisingSSC.cu:512-516), stored as ceil(2^32 p) - 1: a reference
//           uniform (H+1)/2^32 is below p iff H < ceil(2^32 p) - 1;
//   [10,11] MSC thresholds ceil(2^32 e^-4b), ceil(2^32 e^-8b) (PAisingMSC.cu:674-675),
//           also those of the native SSC sweep.
__host__ __device__ inline void thresholds(double beta, uint32_t* t) {
  for (int i0 = 0; i0 <= 1; ++i0)
    for (int i1 = 0; i1 <= 4; ++i1) {
      double p = exp(-2.0 * (2 * i0 - 1) * (2 * i1 - 4) * beta);
      if (p > 1.0) p = 1.0;
      t[i0 + 2 * i1] = (uint32_t)(ceil(4294967296.0 * p) - 1.0);
    }
  const double t4 = ceil(4294967296.0 * exp(-4.0 * beta)), t8 = ceil(4294967296.0 * exp(-8.0 * beta));
  t[10] = t4 >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t4;
  t[11] = t8 >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t8;
}

}  // namespace pa
