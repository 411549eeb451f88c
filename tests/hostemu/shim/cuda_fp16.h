// Host stand-in for the FP16 storage type: IEEE binary16 with
// round-to-nearest-even conversion from float, as __float2half_rn.
#pragma once
#include "cuda_runtime.h"

struct __half {
  _Float16 v;
};
inline float __half2float(__half h) { return (float)h.v; }
inline __half __float2half_rn(float f) { return __half{(_Float16)f}; }
// round toward zero: the nearest value, stepped back one unit when it is larger in magnitude
inline __half __float2half_rz(float f) {
  _Float16 h = (_Float16)f;
  if (__builtin_fabsf((float)h) > __builtin_fabsf(f)) {
    unsigned short bits;
    __builtin_memcpy(&bits, &h, 2);
    bits -= 1;  // same sign, magnitude one unit smaller
    __builtin_memcpy(&h, &bits, 2);
  }
  return __half{h};
}

struct alignas(4) __half2 {
  __half x, y;
};
inline float2 __half22float2(__half2 h) { return float2{(float)h.x.v, (float)h.y.v}; }
