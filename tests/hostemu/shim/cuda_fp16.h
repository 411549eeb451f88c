// Host stand-in for the FP16 storage type: IEEE binary16 with
// round-to-nearest-even conversion from float, as __float2half_rn.
#pragma once
#include "cuda_runtime.h"

struct __half {
  _Float16 v;
};
inline float __half2float(__half h) { return (float)h.v; }
inline __half __float2half_rn(float f) { return __half{(_Float16)f}; }
