// Host stand-ins for the CUDA qualifiers and built-ins used by the flow
// kernels (taxila-lbm_gb300/csrc/tx_kernels.cuh, tx_pair.cuh), so that the
// kernels compile as plain C++ and run one thread at a time on the CPU.  The
// kernels the emulation launches use no shared memory or barriers, so a
// sequential walk over the launch grid computes what the device computes per
// thread (the natural-order conversions, which tile through shared memory,
// are not launched here).  The one warp
// vote (__all_sync, whether a whole warp takes the bounceback-free pushes of
// the paired kernel) sees only the calling thread here: each thread then takes
// that path when it alone qualifies, which the kernel must handle the same.
#pragma once
#include <cstdint>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __launch_bounds__(...)
// parsed only: a kernel that reaches a barrier cannot run one thread at a
// time, so the emulation stops loudly if it ever launches one
#define __shared__ static
[[noreturn]] inline void __syncthreads() { __builtin_trap(); }

struct dim3 {
  unsigned x, y, z;
};
inline dim3 threadIdx, blockIdx, blockDim, gridDim;

struct alignas(8) float2 {
  float x, y;
};
struct alignas(16) float4 {
  float x, y, z, w;
};
struct alignas(8) uint2 {
  unsigned x, y;
};
inline float2 make_float2(float x, float y) { return float2{x, y}; }
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline uint2 make_uint2(unsigned x, unsigned y) { return uint2{x, y}; }
inline unsigned __activemask() { return 0xffffffffu; }
inline bool __all_sync(unsigned, bool p) { return p; }
inline unsigned atomicAdd(unsigned* p, unsigned v) {
  const unsigned o = *p;
  *p = o + v;
  return o;
}
inline float __frcp_rn(float x) { return 1.0f / x; }
inline double __drcp_rn(double x) { return 1.0 / x; }
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
