// Arithmetic-pipe throughput probes: how many FP64 / FP32 instructions per
// second this GPU issues when every warp runs long chains of independent
// operations.  They give the measured compute ceiling that the FP64 step
// kernels are held against (the HBM ceiling is a measured copy bandwidth).
//
// Each thread runs CHAINS (16) independent dependency chains of one operation
// for `iters` iterations (unrolled four times, so that loop bookkeeping is a
// small share of the issued instructions); `blocks` x 256 threads cover the GPU.  The result is
// written out so that nothing is optimised away.  Timed with CUDA events on
// a private stream; the caller samples the SM clock.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int CHAINS = 16;

enum : int { OP_DFMA = 0, OP_DADD = 1, OP_DMUL = 2, OP_FFMA = 3, OP_FFMA2 = 4 };

template <int OP>
__global__ void __launch_bounds__(256) k_pipe(int iters, double b, double c, double* out) {
  const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if constexpr (OP <= OP_DMUL) {
    double a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = 1.0 + 1e-9 * (tid + k);
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < CHAINS; ++k) {
        if constexpr (OP == OP_DFMA) a[k] = fma(a[k], b, c);
        if constexpr (OP == OP_DADD) a[k] = a[k] + c;
        if constexpr (OP == OP_DMUL) a[k] = a[k] * b;
      }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    if (s == 12345.678) out[tid] = s;  // never true for these inputs; keeps the chains live
  } else if constexpr (OP == OP_FFMA) {
    float a[CHAINS];
    const float bf = (float)b, cf = (float)c;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = 1.0f + 1e-6f * (float)(tid + k);
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < CHAINS; ++k) a[k] = fmaf(a[k], bf, cf);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    if (s == 12345.678f) out[tid] = s;
  } else {
    // packed FP32 pairs: each instruction does two FMAs
    float2 a[CHAINS];
    const float2 bf = make_float2((float)b, (float)b), cf = make_float2((float)c, (float)c);
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = make_float2(1.0f + 1e-6f * (float)(tid + k), 1.0f - 1e-6f * (float)k);
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < CHAINS; ++k) a[k] = __ffma2_rn(a[k], bf, cf);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k].x + a[k].y;
    if (s == 12345.678f) out[tid] = s;
  }
}

}  // namespace

extern "C" {

// Runs probe `op` (0 DFMA, 1 DADD, 2 DMUL, 3 FFMA, 4 FFMA2 packed pairs) once
// untimed and `reps` times timed.  *ms: the mean duration of one launch;
// *ops: arithmetic operations of one launch, one per thread instruction
// (threads x iters x chains) and two per packed FFMA2 instruction.
// Returns 0, or the CUDA error code.
int txp_pipe_rate(int op, int blocks, int iters, int reps, double* ms, double* ops) {
  double* out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&out, (size_t)blocks * 256 * sizeof(double));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  auto launch = [&]() {
    const double b = 0.9999999, c = 1e-7;
    switch (op) {
      case OP_DFMA: k_pipe<OP_DFMA><<<blocks, 256, 0, st>>>(iters, b, c, out); break;
      case OP_DADD: k_pipe<OP_DADD><<<blocks, 256, 0, st>>>(iters, b, c, out); break;
      case OP_DMUL: k_pipe<OP_DMUL><<<blocks, 256, 0, st>>>(iters, b, c, out); break;
      case OP_FFMA: k_pipe<OP_FFMA><<<blocks, 256, 0, st>>>(iters, b, c, out); break;
      default: k_pipe<OP_FFMA2><<<blocks, 256, 0, st>>>(iters, b, c, out); break;
    }
  };
  if (e == cudaSuccess && (op < 0 || op > OP_FFMA2 || blocks < 1 || iters < 1 || reps < 1)) e = cudaErrorInvalidValue;
  if (e == cudaSuccess) {
    launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e0, st);
  for (int r = 0; e == cudaSuccess && r < reps; ++r) {
    launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  if (e == cudaSuccess) {
    *ms = (double)t / reps;
    *ops = (double)blocks * 256.0 * (double)iters * CHAINS * (op == OP_FFMA2 ? 2.0 : 1.0);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  return (int)e;
}

}  // extern "C"
