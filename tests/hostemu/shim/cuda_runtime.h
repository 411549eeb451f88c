// Host stand-ins for the CUDA qualifiers and built-ins used by the flow
// kernels (taxila-lbm_gb300/csrc/tx_kernels.cuh), so that the kernels compile
// as plain C++ and run one thread at a time on the CPU.  The kernels use no
// shared memory, barriers, warp operations or atomics, so a sequential walk
// over the launch grid computes exactly what the device computes per thread.
#pragma once
#include <cstdint>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)

struct dim3 {
  unsigned x, y, z;
};
inline dim3 threadIdx, blockIdx, blockDim, gridDim;

struct float2 {
  float x, y;
};
struct alignas(16) double2 {
  double x, y;
};
struct alignas(16) uint4 {
  unsigned x, y, z, w;
};

template <class T>
inline T __ldg(const T* p) {
  return *p;
}

typedef void* cudaStream_t;

inline unsigned __float_as_uint(float f) {
  unsigned u;
  __builtin_memcpy(&u, &f, 4);
  return u;
}
inline float __uint_as_float(unsigned u) {
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
}
