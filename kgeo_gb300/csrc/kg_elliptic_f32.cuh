// FP32 R_C(1, 1 + e) for the mixed-precision sample path (DLMF 19.2.17-20 closed forms, the
// series near e = 0).
#pragma once

#include "kg_common.cuh"

namespace kg {

// R_C(1, 1 + e), e > -1.
KG_HD float rc_one_f(float e) {
  if (fabsf(e) < 2.0e-2f) {
    return 1.0f + e * (-1.0f / 3.0f + e * (1.0f / 5.0f + e * (-1.0f / 7.0f + e * (1.0f / 9.0f + e * (-1.0f / 11.0f)))));
  }
  if (e > 0.0f) {
    float s = sqrtf(e);
    return atanf(s) / s;
  }
  float s = sqrtf(-e);
  return (log1pf(s) - 0.5f * log1pf(e)) / s;
}

}  // namespace kg
